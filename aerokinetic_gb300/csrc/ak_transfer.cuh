// ak_transfer.cuh -- kernels of the two-level (2:1) refined step.
//
// Both levels store pre-collision populations (the reference's
// "collide_stream" order, interface.py:116-130): collide in place, apply the
// boundaries to the post-collision state, then pull-stream into the other
// copy.  The fine level is a padded block (two fine cells of donors around
// the physical fine box in x and y) that wraps in x, y and z; the coarse level
// keeps the uniform engine's layout and legacy outer boundary.
//
// Interface algebra (refinement.py, interface.py, refined_solver.py):
//   moments      (rho, j, Pi_neq) of 27 populations, with the reference's
//                positivity and Mach <= 0.3 checks (a failed check sets a flag)
//   populations  tensor-product equilibrium + second-order Hermite stress
//   prolongation per axis children = parent -+ [11/64 (a+1 - a-1) - 3/128 (a+2 - a-2)]
//   restriction  mean of the 2x2x2 children
//   rescale      stress scaled by tau dt ratios (shear / bulk separately)
//   face fluxes  exact moment flux of pull streaming through a face patch,
//                diagonal links split over axis orderings
// All interface arithmetic is FP64 whatever the population storage.
#pragma once
#include <type_traits>

#include "ak_kernels.cuh"

namespace ak {

constexpr double TCS2 = 1.0 / 3.0;
// second-order index pairs (xx, yy, zz, xy, xz, yz)
__host__ __device__ constexpr int sa(int k) { return k < 3 ? k : (k == 5 ? 1 : 0); }
__host__ __device__ constexpr int sb(int k) { return k < 3 ? k : (k == 3 ? 1 : 2); }

// error flags of the transfer checks
constexpr int XF_DENSITY = 1, XF_NEGATIVE = 2, XF_MACH = 4, XF_NONFINITE = 8;

// compile-time loop: f(std::integral_constant<int, i>) for i in [B, E)
template <int B, int E, typename F>
__device__ __forceinline__ void static_for(F &&f) {
    if constexpr (B < E) {
        f(std::integral_constant<int, B>{});
        static_for<B + 1, E>(f);
    }
}

// The transfer algebra runs in the storage form's arithmetic type T: FP64 for
// the plain form, FP32 for the FP32-compute forms.

// running sums of one cell: drho, j (3), second moments (xx, yy, zz, xy, xz, yz);
// the zero products of the lattice velocities are skipped
template <int q, typename T>
__device__ __forceinline__ void add_moments(T s[10], T v) {
    constexpr int c[3] = {cx(q), cy(q), cz(q)};
    s[0] += v;
#pragma unroll
    for (int a = 0; a < 3; ++a)
        if (c[a] != 0) s[1 + a] += c[a] > 0 ? v : -v;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const int p = c[sa(k)] * c[sb(k)];
        if (p != 0) s[4 + k] += p > 0 ? v : -v;
    }
}

// the same sums of one cell from all 27 of its populations, reduced axis by
// axis (x moments of each (cy, cz) line, then y, then z): 68 additions
// instead of the 171 of add_moments over every direction
template <typename T>
__host__ __device__ __forceinline__ void cell_moments(const T g[Q], T s[10]) {
    T a0[3][3], a1[3][3], a2[3][3];  // [cy + 1][cz + 1]: sum, sum cx, sum cx^2
#pragma unroll
    for (int iy = 0; iy < 3; ++iy)
#pragma unroll
        for (int iz = 0; iz < 3; ++iz) {
            const T m = g[qof(0, iy, iz)], o = g[qof(1, iy, iz)], p = g[qof(2, iy, iz)];
            a2[iy][iz] = p + m;
            a1[iy][iz] = p - m;
            a0[iy][iz] = a2[iy][iz] + o;
        }
    // per cz: sum, sum cy, sum cy^2 of a0; sum, sum cy of a1; sum of a2
    T b00[3], b01[3], b02[3], b10[3], b11[3], b20[3];
#pragma unroll
    for (int iz = 0; iz < 3; ++iz) {
        b02[iz] = a0[2][iz] + a0[0][iz];
        b01[iz] = a0[2][iz] - a0[0][iz];
        b00[iz] = b02[iz] + a0[1][iz];
        b11[iz] = a1[2][iz] - a1[0][iz];
        b10[iz] = (a1[2][iz] + a1[0][iz]) + a1[1][iz];
        b20[iz] = (a2[2][iz] + a2[0][iz]) + a2[1][iz];
    }
    const T zz = b00[2] + b00[0];
    s[0] = zz + b00[1];
    s[1] = (b10[2] + b10[0]) + b10[1];
    s[2] = (b01[2] + b01[0]) + b01[1];
    s[3] = b00[2] - b00[0];
    s[4] = (b20[2] + b20[0]) + b20[1];  // xx
    s[5] = (b02[2] + b02[0]) + b02[1];  // yy
    s[6] = zz;                          // zz
    s[7] = (b11[2] + b11[0]) + b11[1];  // xy
    s[8] = b10[2] - b10[0];             // xz
    s[9] = b01[2] - b01[0];             // yz
}

// (rho, j, Pi_neq) from the running sums, with the reference's density and
// Mach <= 0.3 checks (refinement.py:140-173); report = 0 skips the checks.
// The Mach test compares |j|^2 with (0.3 c_s rho)^2 (same decision up to the
// rounding of the threshold) and the stress divides by rho through one
// reciprocal: the FP64 pipe is the limit of these kernels.
template <typename T>
__device__ __forceinline__ void finish_moments(const T s[10], T m[10], int *flag, bool report) {
    const T drho = s[0], rho = drho + T(1), inv = T(1) / rho;
    if (report) {
        if (!(rho > T(0))) atomicOr(flag, XF_DENSITY);
        if (s[1] * s[1] + s[2] * s[2] + s[3] * s[3] > T(0.09 * TCS2) * rho * rho) atomicOr(flag, XF_MACH);
    }
    m[0] = rho;
    m[1] = s[1];
    m[2] = s[2];
    m[3] = s[3];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        T p = s[4 + k];
        if (k < 3) p -= drho * T(TCS2);
        m[4 + k] = p - s[1 + sa(k)] * s[1 + sb(k)] * inv;
    }
}

// checks of a moment set before populations are built from it
template <typename T>
__device__ __forceinline__ void check_fields(const T m[10], int *flag) {
    const T rho = m[0];
    if (!(rho > T(0))) atomicOr(flag, XF_DENSITY);
    if (m[1] * m[1] + m[2] * m[2] + m[3] * m[3] > T(0.09 * TCS2) * rho * rho) atomicOr(flag, XF_MACH);
}

// per-axis factors of the tensor-product equilibrium, fac[a][c + 1]:
// 2/3 - u^2 for c = 0, (1/3 + u^2 + c u) / 2 otherwise
template <typename T>
__device__ __forceinline__ void axis_factors(const T m[10], T fac[9]) {
    const T inv = T(1) / m[0];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const T u = m[1 + a] * inv, uu = u * u;
        fac[3 * a + 0] = (T(TCS2) + uu - u) / T(2);
        fac[3 * a + 1] = T(2.0 / 3.0) - uu;
        fac[3 * a + 2] = (T(TCS2) + uu + u) / T(2);
    }
}

// zero-centred population q of (rho, j, Pi_neq) (refinement.py:177-203):
// tensor-product equilibrium + second-order Hermite stress term
template <int q, typename T>
__device__ __forceinline__ T population(const T m[10], const T fac[9], bool &bad) {
    constexpr int c[3] = {cx(q), cy(q), cz(q)};
    T eq = fac[c[0] + 1] * fac[3 + c[1] + 1];
    eq *= fac[6 + c[2] + 1];
    eq *= m[0];
    T neq = 0;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        double h = (double)(c[sa(k)] * c[sb(k)]) - (k < 3 ? TCS2 : 0.0);
        if (k >= 3) h *= 2.0;
        if (h != 0.0) neq += T(weight(q) * h / (2.0 * TCS2 * TCS2)) * m[4 + k];
    }
    const T f = eq + neq;
    bad |= !isfinite(f) || f < T(0);
    return f - T(weight(q));
}

// ------------------------------------------------------------ direction-split blocks
// The interface kernels run 256-thread blocks over 32 cells: the lane is the
// cell slot (consecutive x, so every direction plane is read coalesced) and
// warp w owns the directions w, w + 8, w + 16 (and w + 24 < 27) with
// compile-time indices.  Per-cell sums cross the warps through shared memory
// in a fixed order, so results do not depend on scheduling.
constexpr int SPLIT_THREADS = 256, SPLIT_CELLS = 32, SPLIT_WARPS = 8;

template <typename F>
__device__ __forceinline__ void by_warp(F &&f) {
    switch (threadIdx.x >> 5) {
    case 0: f(std::integral_constant<int, 0>{}); break;
    case 1: f(std::integral_constant<int, 1>{}); break;
    case 2: f(std::integral_constant<int, 2>{}); break;
    case 3: f(std::integral_constant<int, 3>{}); break;
    case 4: f(std::integral_constant<int, 4>{}); break;
    case 5: f(std::integral_constant<int, 5>{}); break;
    case 6: f(std::integral_constant<int, 6>{}); break;
    default: f(std::integral_constant<int, 7>{}); break;
    }
}

// f(integral_constant<q>, slot) over the directions owned by warp W
template <int W, typename F>
__device__ __forceinline__ void owned(F &&f) {
    f(std::integral_constant<int, W>{}, 0);
    f(std::integral_constant<int, W + 8>{}, 1);
    f(std::integral_constant<int, W + 16>{}, 2);
    if constexpr (W + 24 < Q) f(std::integral_constant<int, W + 24>{}, 3);
}

// shared state of a direction-split block: per-warp partial sums and the
// per-cell fields (moments + equilibrium factors) that warp 0 prepares
constexpr int NFIELD = 19;  // m[10], fac[9]
template <typename T>
struct SplitShared {
    T part[SPLIT_WARPS][10][SPLIT_CELLS];
    int neg[SPLIT_WARPS][SPLIT_CELLS];
    T field[2][NFIELD][SPLIT_CELLS];
};

template <typename T>
__device__ __forceinline__ void put_partial(SplitShared<T> &sh, const T s[10], bool neg) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 10; ++k) sh.part[w][k][lane] = s[k];
    sh.neg[w][lane] = neg;
}
// block-wide sums of the cell slot, warps 0..7 in order (after a barrier)
template <typename T>
__device__ __forceinline__ void sum_partials(const SplitShared<T> &sh, T t[10], bool &any_neg) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < 10; ++k) {
        T v = sh.part[0][k][lane];
#pragma unroll
        for (int j = 1; j < SPLIT_WARPS; ++j) v += sh.part[j][k][lane];
        t[k] = v;
    }
    any_neg = false;
#pragma unroll
    for (int j = 0; j < SPLIT_WARPS; ++j) any_neg |= sh.neg[j][lane] != 0;
}
template <typename T>
__device__ __forceinline__ void put_fields(SplitShared<T> &sh, int set, const T m[10]) {
    const int lane = threadIdx.x & 31;
    T fac[9];
    axis_factors(m, fac);
#pragma unroll
    for (int k = 0; k < 10; ++k) sh.field[set][k][lane] = m[k];
#pragma unroll
    for (int k = 0; k < 9; ++k) sh.field[set][10 + k][lane] = fac[k];
}
template <typename T>
__device__ __forceinline__ void get_fields(const SplitShared<T> &sh, int set, T m[10], T fac[9]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < 10; ++k) m[k] = sh.field[set][k][lane];
#pragma unroll
    for (int k = 0; k < 9; ++k) fac[k] = sh.field[set][10 + k][lane];
}

// a population in the arithmetic type T of its storage form
template <typename T, typename S>
__device__ __forceinline__ T load_as(const S *pdf, const Grid &G, int q, int x, int y, int z) {
    if (!AK_CHECK(G, q, x, y, z, 1)) return T(0);
    return (T)Store<S>::load(pdf + q * G.qs + G.cell(x, y, z), q, G.shift[q]);
}
template <typename T, typename S>
__device__ __forceinline__ void store_as(S *pdf, const Grid &G, int q, int x, int y, int z, T v) {
    if (!AK_CHECK(G, q, x, y, z, 2)) return;
    Store<S>::store(pdf + q * G.qs + G.cell(x, y, z), q, (typename Store<S>::T)v, G.shift[q]);
}

// cells of an nx x ny rectangle outside its interior [wx, nx - wx) x
// [wy, ny - wy) (the whole rectangle when no interior is left): the count,
// and the b-th cell, rows first
__host__ __device__ __forceinline__ long long ring_count(int nx, int ny, int wx, int wy) {
    if (nx <= 2 * wx || ny <= 2 * wy) return (long long)nx * ny;
    return 2LL * wy * nx + 2LL * wx * (ny - 2 * wy);
}
__device__ __forceinline__ void ring_cell(long long b, int nx, int ny, int wx, int wy, int &x, int &y) {
    if (nx <= 2 * wx || ny <= 2 * wy) {
        y = (int)(b / nx);
        x = (int)(b - (long long)y * nx);
        return;
    }
    const long long rows = (long long)wy * nx;
    if (b < 2 * rows) {
        const int r = (int)(b / nx);
        x = (int)(b - (long long)r * nx);
        y = r < wy ? r : ny - 2 * wy + r;
        return;
    }
    b -= 2 * rows;
    const int r = (int)(b / (2 * wx)), k = (int)(b - (long long)r * 2 * wx);
    y = wy + r;
    x = k < wx ? k : nx - 2 * wx + k;
}

struct Rescale {
    double shear, bulk;  // target tau dt / source tau dt
};
template <typename T>
__device__ __forceinline__ void rescale_stress(T m[10], Rescale r) {
    const T iso = (m[4] + m[5] + m[6]) / T(3);
#pragma unroll
    for (int k = 4; k < 10; ++k) m[k] *= T(r.shear);
#pragma unroll
    for (int k = 4; k < 7; ++k) m[k] += T(r.bulk - r.shear) * iso;
}

// ------------------------------------------------------------ split step
template <typename S>
__global__ void __launch_bounds__(128, Store<S>::MIN_BLOCKS)
    k_collide(S *__restrict__ pdf, const uint8_t *__restrict__ flags, Grid G, Shift27 shift,
              typename Store<S>::T omega_s, typename Store<S>::T omega_b,
              int4 rect = make_int4(0, 0, 0, 0), int4 skip = make_int4(0, 0, 0, 0)) {
    chain_wait();
    using T = typename Store<S>::T;
    // one thread per cell of the padded columns x [rect.x, rect.y) by y
    // [rect.z, rect.w) (rect.y == 0: the whole interior), every z, x fastest,
    // numbered across rows: warps stay full whatever the width (this kernel is
    // bound by the FP64 pipe in the plain form, where a warp with a few live
    // lanes costs a full one); columns inside skip are left as they are
    if (rect.y == 0) rect = make_int4(1, G.nx + 1, 1, G.ny + 1);
    const unsigned w = (unsigned)(rect.y - rect.x), h = (unsigned)(rect.w - rect.z);
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned nxy = w * h;
    if (i >= nxy * (unsigned)G.nz) return;
    const unsigned z = i / nxy, r = i - z * nxy;
    const unsigned yr = r / w;
    const int x = rect.x + (int)(r - yr * w), y = rect.z + (int)yr;
    if (x >= skip.x && x < skip.y && y >= skip.z && y < skip.w) return;
    if (__ldg(flags + y * G.nxp + x) != FLAG_FLUID) return;
    const long long c = G.cell(x, y, z);
    T g[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) g[q] = Store<S>::load(pdf + q * G.qs + c, q, shift.v[q]);
    collide_stored<S>(g, omega_s, omega_b);
#pragma unroll
    for (int q = 0; q < Q; ++q) Store<S>::store(pdf + q * G.qs + c, q, g[q], shift.v[q]);
}

// the collision of the cells of the padding band (pad cells around the
// physical block in x and y, every z) alone, numbered around the ring so
// that every lane of a warp holds a band cell
template <typename S>
__global__ void __launch_bounds__(128, Store<S>::MIN_BLOCKS)
    k_collide_band(S *__restrict__ pdf, const uint8_t *__restrict__ flags, Grid G, Shift27 shift,
                   typename Store<S>::T omega_s, typename Store<S>::T omega_b, int pad) {
    chain_wait();
    using T = typename Store<S>::T;
    const long long nring = ring_count(G.nx, G.ny, pad, pad);
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nring * G.nz) return;
    const int z = (int)(i / nring);
    int x, y;
    ring_cell(i - z * nring, G.nx, G.ny, pad, pad, x, y);
    if (__ldg(flags + (y + 1) * G.nxp + x + 1) != FLAG_FLUID) return;
    const long long c = G.cell(x + 1, y + 1, z);
    T g[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) g[q] = Store<S>::load(pdf + q * G.qs + c, q, shift.v[q]);
    collide_stored<S>(g, omega_s, omega_b);
#pragma unroll
    for (int q = 0; q < Q; ++q) Store<S>::store(pdf + q * G.qs + c, q, g[q], shift.v[q]);
}

// pull streaming of the stored values (bit copies); x and y wrap when periodic
template <typename S>
__global__ void k_stream(const S *__restrict__ src, S *__restrict__ dst, const uint8_t *__restrict__ flags, Grid G,
                         int periodic_xy) {
    chain_wait();
    const int x = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int y = blockIdx.y + 1;
    const int z = blockIdx.z;
    if (x > G.nx) return;
    if (__ldg(flags + y * G.nxp + x) != FLAG_FLUID) return;
    const long long c = G.cell(x, y, z);
    if (!periodic_xy) {
        // the cell's column in the three z planes it pulls from: one address
        // add per population
        const S *row[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) row[k] = src + (long long)G.wrapz(z - (k - 1)) * G.plane + (long long)y * G.sx + x;
#pragma unroll
        for (int q = 0; q < Q; ++q)
            dst[q * G.qs + c] = row[cz(q) + 1][(long long)q * G.qs - (long long)cy(q) * G.sx - cx(q)];
        return;
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        int xs = x - cx(q), ys = y - cy(q);
        xs = xs < 1 ? xs + G.nx : (xs > G.nx ? xs - G.nx : xs);
        ys = ys < 1 ? ys + G.ny : (ys > G.ny ? ys - G.ny : ys);
        dst[q * G.qs + c] = src[q * G.qs + G.cell(xs, ys, G.wrapz(z - cz(q)))];
    }
}

// The pre-collision coarse state of the fused form, (x, y, z, 27) doubles:
// mode 1 (after a step) pulls every cell outside the transfer block (padded
// columns x [xfer.x, xfer.y) by y [xfer.z, xfer.w)) from the other copy,
// which the step's fused pass read with the outer boundaries applied, and
// takes the transfer block's cells from the current copy; mode 0 (after
// set-up) reads every cell of the other copy.
template <typename S>
__global__ void k_export_pre_collision(const S *__restrict__ cur, const S *__restrict__ other, Grid G, int4 xfer,
                                       int mode, double *__restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)G.nx * G.ny * G.nz) return;
    const int z = (int)(i % G.nz);
    const long long xy = i / G.nz;
    const int y = (int)(xy % G.ny) + 1, x = (int)(xy / G.ny) + 1;
    const bool block = x >= xfer.x && x < xfer.y && y >= xfer.z && y < xfer.w;
    for (int q = 0; q < Q; ++q) {
        double v;
        if (mode == 0)
            v = load_g(other, G, q, x, y, z);
        else if (block)
            v = load_g(cur, G, q, x, y, z);
        else
            v = load_g(other, G, q, x - cx(q), y - cy(q), G.wrapz(z - cz(q)));
        out[i * Q + q] = v;
    }
}

// every cell, ghosts included, set to the given zero-centred populations
template <typename S>
__global__ void k_fill(S *__restrict__ pdf, Grid G, const double *__restrict__ g27) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= G.qs) return;
    const int z = (int)(i / G.plane);
    const long long r = i - (long long)z * G.plane;
    const int y = (int)(r / G.sx), x = (int)(r - (long long)y * G.sx);
    if (x >= G.nxp) return;
    for (int q = 0; q < Q; ++q) store_g(pdf, G, q, x, y, z, g27[q]);
}

// ------------------------------------------------------------ face fluxes
struct FluxTerm {
    int d;          // direction
    int shift[3];   // tangential shift of the source cell (-c_a on the moved axes)
    double coef[4]; // weight * normal * (1, c)
};

struct Face {
    int axis, side;       // normal axis; -1 lower face of the box, +1 upper
    int lo1, lo2, n1, n2; // tangential start (interior coordinates) and extent, coarse units
    int coarse_index;     // face index on the coarse lattice (upper face of that cell)
    int fine_index;       // face index on the fine lattice (interior coordinates of the padded block)
};

// one term of a face patch entry at lattice coordinates p1, p2 (interior)
template <typename S>
__device__ __forceinline__ void face_term_add(const S *pdf, const Grid &G, const FluxTerm &T, int axis, int index,
                                              int p1, int p2, bool periodic, double acc[4]) {
    const int a1 = axis == 0 ? 1 : 0, a2 = axis == 2 ? 1 : 2;
    const int dims[3] = {G.nx, G.ny, G.nz};
    const int normal = axis == 0 ? cx(T.d) : (axis == 1 ? cy(T.d) : cz(T.d));
    int c3[3];
    c3[axis] = index + (normal < 0 ? 1 : 0);
    c3[a1] = p1 + T.shift[a1];
    c3[a2] = p2 + T.shift[a2];
    if (periodic) {
        for (int a = 0; a < 3; ++a) c3[a] = (c3[a] % dims[a] + dims[a]) % dims[a];
    } else {
        c3[2] = (c3[2] % dims[2] + dims[2]) % dims[2];
    }
    const double v = load_g(pdf, G, T.d, c3[0] + 1, c3[1] + 1, c3[2]);
    for (int k = 0; k < 4; ++k) acc[k] += v * T.coef[k];
}

__device__ __forceinline__ void warp_sum4(double acc[4]) {
    for (int o = 16; o > 0; o >>= 1)
        for (int k = 0; k < 4; ++k) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], o);
}

// coarse faces: reg[face][t1][t2][4] = flux * dx^3; one warp per entry
template <typename S>
__global__ void k_face_flux_coarse(const S *__restrict__ pdf, Grid G, const FluxTerm *__restrict__ terms0,
                                   const FluxTerm *__restrict__ terms1, int nterms, const Face *__restrict__ faces,
                                   int nfaces, const long long *__restrict__ offsets, double scale,
                                   double *__restrict__ reg) {
    const int f = blockIdx.y;
    if (f >= nfaces) return;
    const Face F = faces[f];
    const long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= (long long)F.n1 * F.n2) return;
    const int t1 = (int)(i / F.n2), t2 = (int)(i - (long long)t1 * F.n2);
    const FluxTerm *terms = F.axis == 0 ? terms0 : terms1;
    double acc[4] = {0, 0, 0, 0};
    for (int t = lane; t < nterms; t += 32)
        face_term_add(pdf, G, terms[t], F.axis, F.coarse_index, F.lo1 + t1, F.lo2 + t2, true, acc);
    warp_sum4(acc);
    if (lane == 0) {
        double *r = reg + offsets[f] + 4 * i;
        for (int k = 0; k < 4; ++k) r[k] = acc[k] * scale;
    }
}

// fine faces: each coarse entry accumulates the sum of its 2 x 2 fine
// entries; one warp per coarse entry
template <typename S>
__global__ void k_face_flux_fine(const S *__restrict__ pdf, Grid G, const FluxTerm *__restrict__ terms0,
                                 const FluxTerm *__restrict__ terms1, int nterms, const Face *__restrict__ faces,
                                 int nfaces, const long long *__restrict__ offsets, int pad, double scale,
                                 double *__restrict__ reg) {
    const int f = blockIdx.y;
    if (f >= nfaces) return;
    const Face F = faces[f];
    const long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= (long long)F.n1 * F.n2) return;
    const int t1 = (int)(i / F.n2), t2 = (int)(i - (long long)t1 * F.n2);
    // fine tangential origin: x and y start after the donor padding, z at 0
    const int a1 = F.axis == 0 ? 1 : 0, a2 = F.axis == 2 ? 1 : 2;
    const int o1 = a1 < 2 ? pad : 0, o2 = a2 < 2 ? pad : 0;
    const FluxTerm *terms = F.axis == 0 ? terms0 : terms1;
    double acc[4] = {0, 0, 0, 0};
    for (int item = lane; item < 4 * nterms; item += 32) {
        const int sub = item / nterms, t = item - sub * nterms;
        face_term_add(pdf, G, terms[t], F.axis, F.fine_index, o1 + 2 * t1 + (sub & 1), o2 + 2 * t2 + (sub >> 1),
                      false, acc);
    }
    warp_sum4(acc);
    if (lane == 0) {
        double *r = reg + offsets[f] + 4 * i;
        for (int k = 0; k < 4; ++k) r[k] += acc[k] * scale;
    }
}

// ------------------------------------------------------------ donors
struct BoxSpec {
    int lo[3], hi[3];  // fine box in coarse cells
    int bx, by, bz;    // box extent
    int dx0, dy0;      // donor block origin in coarse x, y (lo - 3)
    int dnx, dny;      // donor block extent in x, y (b + 6); z covers the whole span
};

__device__ __forceinline__ bool in_core(const BoxSpec &B, int cxi, int cyi) {
    // covered coarse cell more than three cells inside the box (x and y)
    return cxi >= B.lo[0] + 3 && cxi < B.hi[0] - 3 && cyi >= B.lo[1] + 3 && cyi < B.hi[1] - 3;
}

// Moments of the donor block: coarse cells [lo-3, hi+3) in x and y (periodic
// wrap, as the reference indexes them), all z; covered core cells take the
// free-stream populations.  Output out[k][z][y][x] (x fastest, n cells),
// written on the ring of the block the prolongation reads (five cells wide);
// with mix_from set, half also receives 0.5 mix_from + 0.5 out, the donor
// moments half-way through the coarse step.  Moments and their prolongation
// are held in the transfer arithmetic type T of the storage form.
constexpr int DONOR_RING = 5;
template <typename S>
__global__ void __launch_bounds__(SPLIT_THREADS)
    k_block_moments(const S *__restrict__ pdf, Grid G, BoxSpec B, const double *__restrict__ free_g,
                    typename Store<S>::A *__restrict__ out, const typename Store<S>::A *__restrict__ mix_from,
                    typename Store<S>::A *__restrict__ half, int *__restrict__ flag) {
    chain_wait();
    using T = typename Store<S>::A;
    __shared__ SplitShared<T> sh;
    const long long nring = ring_count(B.dnx, B.dny, DONOR_RING, DONOR_RING), nr = nring * G.nz;
    if ((long long)blockIdx.x * SPLIT_CELLS >= nr) return;
    const int lane = threadIdx.x & 31;
    const long long i = (long long)blockIdx.x * SPLIT_CELLS + lane;
    const bool valid = i < nr;
    int bx = 0, by = 0, z = 0, cxi = 0, cyi = 0;
    bool core = false;
    if (valid) {
        z = (int)(i / nring);
        ring_cell(i - z * nring, B.dnx, B.dny, DONOR_RING, DONOR_RING, bx, by);
        cxi = ((B.dx0 + bx) % G.nx + G.nx) % G.nx;
        cyi = ((B.dy0 + by) % G.ny + G.ny) % G.ny;
        core = in_core(B, cxi, cyi);
    }
    T s[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    bool neg = false;
    by_warp([&](auto wc) {
        owned<decltype(wc)::value>([&](auto qc, int) {
            constexpr int q = decltype(qc)::value;
            T v = 0;
            if (valid) v = core ? T(free_g[q]) : load_as<T>(pdf, G, q, cxi + 1, cyi + 1, z);
            add_moments<q>(s, v);
            neg |= v < T(-weight(q));
        });
    });
    put_partial(sh, s, neg);
    __syncthreads();
    if ((threadIdx.x >> 5) != 0 || !valid) return;
    T t[10], m[10];
    bool any_neg;
    sum_partials(sh, t, any_neg);
    if (any_neg) atomicOr(flag, XF_NEGATIVE);
    finish_moments(t, m, flag, true);
    const long long n = (long long)B.dnx * B.dny * G.nz, j = ((long long)z * B.dny + by) * B.dnx + bx;
#pragma unroll
    for (int k = 0; k < 10; ++k) {
        out[k * n + j] = m[k];
        if (mix_from) half[k * n + j] = T(0.5) * mix_from[k * n + j] + T(0.5) * m[k];
    }
}

// Donors for the padding band of the fine block: the donor moments are
// prolonged one axis at a time, as the reference does (refinement.py:78-105):
// children = centre -+ [11/64 (a+1 - a-1) - 3/128 (a+2 - a-2)].
template <typename T>
__device__ __forceinline__ T prolong_child(T am2, T am1, T a0, T ap1, T ap2, int odd) {
    const T offset = T(11.0 / 64.0) * (ap1 - am1) - T(3.0 / 128.0) * (ap2 - am2);
    return odd ? a0 + offset : a0 - offset;
}

// x pass: out[k][z][by][fx] (fx fastest, fx in [0, nfx = 2 (bx + 2))), on the
// cells the y pass reads for the band: every fx of the five outer block rows
// on each side, the band columns elsewhere
template <typename T>
__global__ void k_prolong_x(BoxSpec B, int nz, int pad, const T *__restrict__ m, T *__restrict__ out) {
    chain_wait();
    const int nfx = 2 * (B.bx + 2);
    const long long nring = ring_count(nfx, B.dny, pad, DONOR_RING);
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nring * nz) return;
    const int z = (int)(i / nring);
    int fx, by;
    ring_cell(i - z * nring, nfx, B.dny, pad, DONOR_RING, fx, by);
    const long long n = (long long)nfx * B.dny * nz, nblock = (long long)B.dnx * B.dny * nz;
    const long long row = (long long)z * B.dny + by, o = row * nfx + fx, base = row * B.dnx + (fx >> 1);
#pragma unroll
    for (int k = 0; k < 10; ++k) {
        const T *a = m + k * nblock + base;
        out[k * n + o] = prolong_child(a[0], a[1], a[2], a[3], a[4], fx & 1);
    }
}

// y and z passes on the padding band (pad fine cells around the physical
// block in x and y, every z), stress rescaled coarse -> fine, populations.
// Warp w prolongs moments w and w + 8: each of the five coarse z planes the
// z pass reads is first prolonged in y from the x pass's rows, so the y pass
// needs no launch of its own (the same operations on the same values).  Warp
// 0 rescales and prepares the fields, every warp writes its own directions.
// COLLIDE: the populations go through shared memory instead, and warp 0
// collides its 32 fluid cells (as k_collide would, on the values the storage
// would hold) and stores the post-collision populations.  Forms whose stored
// value is not the computed one (FP16) are not compiled with it.
template <typename S, bool COLLIDE = false>
__global__ void __launch_bounds__(SPLIT_THREADS)
    k_donors(S *__restrict__ fine, Grid F, int nzc, const typename Store<S>::A *__restrict__ px, int dny, Rescale r,
             int pad, int *__restrict__ flag, const uint8_t *__restrict__ flags = nullptr,
             typename Store<S>::T omega_s = 0, typename Store<S>::T omega_b = 0) {
    static_assert(!COLLIDE || !std::is_same_v<S, __half>, "FP16 storage rounds the donors before the collision");
    chain_wait();
    using T = typename Store<S>::A;
    __shared__ SplitShared<T> sh;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const long long nring = ring_count(F.nx, F.ny, pad, pad), n = nring * F.nz;
    if ((long long)blockIdx.x * SPLIT_CELLS >= n) return;
    const long long i = (long long)blockIdx.x * SPLIT_CELLS + lane;
    const bool valid = i < n;
    int fx = 0, fy = 0, fz = 0;
    if (valid) {
        fz = (int)(i / nring);
        ring_cell(i - fz * nring, F.nx, F.ny, pad, pad, fx, fy);
    }
    // x-pass rows: px[k][z][by][fx], fx in [0, F.nx), by in [0, dny)
    const long long nin = (long long)F.nx * dny * nzc, row0 = (long long)(fy >> 1) * F.nx + fx;
    const int pz = fz >> 1;
    for (int k = w; k < 10; k += SPLIT_WARPS) {
        T a[5];
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            const int zz = ((pz + j - 2) % nzc + nzc) % nzc;
            if (valid) {
                const T *b = px + k * nin + (long long)zz * dny * F.nx + row0;
                a[j] = prolong_child(b[0], b[F.nx], b[2 * F.nx], b[3 * F.nx], b[4 * F.nx], fy & 1);
            } else {
                a[j] = k == 0 ? T(1) : T(0);
            }
        }
        sh.field[0][k][lane] = prolong_child(a[0], a[1], a[2], a[3], a[4], fz & 1);
    }
    __syncthreads();
    if (w == 0) {
        T m[10];
#pragma unroll
        for (int k = 0; k < 10; ++k) m[k] = sh.field[0][k][lane];
        rescale_stress(m, r);
        if (valid) check_fields(m, flag);
        put_fields(sh, 1, m);
    }
    __syncthreads();
    T m[10], fac[9];
    get_fields(sh, 1, m, fac);
    bool bad = false;
    if constexpr (COLLIDE) {
        __shared__ T pop[Q][SPLIT_CELLS];
        by_warp([&](auto wc) {
            owned<decltype(wc)::value>([&](auto qc, int) {
                constexpr int q = decltype(qc)::value;
                pop[q][lane] = population<q>(m, fac, bad);
            });
        });
        if (bad && valid) atomicOr(flag, XF_NEGATIVE);
        __syncthreads();
        if (w != 0 || !valid) return;
        using TS = typename Store<S>::T;
        TS g[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) g[q] = TS(pop[q][lane]);
        if (__ldg(flags + (fy + 1) * F.nxp + fx + 1) == FLAG_FLUID) collide_stored<S>(g, omega_s, omega_b);
        const long long c = F.cell(fx + 1, fy + 1, fz);
#pragma unroll
        for (int q = 0; q < Q; ++q)
            if (AK_CHECK(F, q, fx + 1, fy + 1, fz, 2)) Store<S>::store(fine + q * F.qs + c, q, g[q], F.shift[q]);
    } else {
        by_warp([&](auto wc) {
            owned<decltype(wc)::value>([&](auto qc, int) {
                constexpr int q = decltype(qc)::value;
                const T g = population<q>(m, fac, bad);
                if (valid) store_as<T>(fine, F, q, fx + 1, fy + 1, fz, g);
            });
        });
        if (bad && valid) atomicOr(flag, XF_NEGATIVE);
    }
}

// ------------------------------------------------------------ reflux, restriction
// coarse cells just outside each face: equilibrium part of the state shifted
// by the flux mismatch (interface.py:285-295)
template <typename S>
__global__ void __launch_bounds__(SPLIT_THREADS)
    k_reflux(S *__restrict__ pdf, Grid G, const Face *__restrict__ faces, int nfaces,
             const long long *__restrict__ offsets, const double *__restrict__ reg_c,
             const double *__restrict__ reg_f, double inv_volume, int *__restrict__ flag) {
    chain_wait();
    using T = typename Store<S>::A;
    __shared__ SplitShared<T> sh;
    const int f = blockIdx.y;
    if (f >= nfaces) return;
    const Face F = faces[f];
    const long long n = (long long)F.n1 * F.n2;
    if ((long long)blockIdx.x * SPLIT_CELLS >= n) return;
    const int lane = threadIdx.x & 31;
    const bool lead = (threadIdx.x >> 5) == 0;
    const long long i = (long long)blockIdx.x * SPLIT_CELLS + lane;
    const bool valid = i < n;
    const long long e = valid ? i : 0;
    const int t1 = (int)(e / F.n2), t2 = (int)(e - (long long)t1 * F.n2);
    const int a1 = F.axis == 0 ? 1 : 0, a2 = F.axis == 2 ? 1 : 2;
    int c3[3];
    c3[F.axis] = F.side < 0 ? F.coarse_index : F.coarse_index + 1;  // the cell outside the box
    c3[a1] = F.lo1 + t1;
    c3[a2] = F.lo2 + t2;
    T g[4] = {0, 0, 0, 0}, s[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    bool neg = false;
    by_warp([&](auto wc) {
        owned<decltype(wc)::value>([&](auto qc, int slot) {
            constexpr int q = decltype(qc)::value;
            g[slot] = valid ? load_as<T>(pdf, G, q, c3[0] + 1, c3[1] + 1, c3[2]) : T(0);
            add_moments<q>(s, g[slot]);
            neg |= g[slot] < T(-weight(q));
        });
    });
    put_partial(sh, s, neg);
    __syncthreads();
    if (lead) {
        T t[10], m_old[10], m_new[10];
        bool any_neg;
        sum_partials(sh, t, any_neg);
        if (valid && any_neg) atomicOr(flag, XF_NEGATIVE);
        finish_moments(t, m_old, flag, valid);
        const double *rc = reg_c + offsets[f] + 4 * e, *rf = reg_f + offsets[f] + 4 * e;
#pragma unroll
        for (int k = 4; k < 10; ++k) m_old[k] = T(0);
#pragma unroll
        for (int k = 0; k < 10; ++k) m_new[k] = m_old[k];
#pragma unroll
        for (int k = 0; k < 4; ++k) m_new[k] += T(F.side * (rf[k] - rc[k]) * inv_volume);
        if (valid) {
            check_fields(m_new, flag);
            check_fields(m_old, flag);
        }
        put_fields(sh, 0, m_new);
        put_fields(sh, 1, m_old);
    }
    __syncthreads();
    T m_new[10], f_new[9], m_old[10], f_old[9];
    get_fields(sh, 0, m_new, f_new);
    get_fields(sh, 1, m_old, f_old);
    bool bad = false, neg2 = false;
    T s2[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    by_warp([&](auto wc) {
        owned<decltype(wc)::value>([&](auto qc, int slot) {
            constexpr int q = decltype(qc)::value;
            g[slot] += population<q>(m_new, f_new, bad) - population<q>(m_old, f_old, bad);
            add_moments<q>(s2, g[slot]);
            neg2 |= g[slot] < T(-weight(q));
            if (valid) store_as<T>(pdf, G, q, c3[0] + 1, c3[1] + 1, c3[2], g[slot]);
        });
    });
    if (bad && valid) atomicOr(flag, XF_NEGATIVE);
    // the shifted state passes the same checks (interface.py:293)
    __syncthreads();
    put_partial(sh, s2, neg2);
    __syncthreads();
    if (lead && valid) {
        T t[10], chk[10];
        bool any_neg;
        sum_partials(sh, t, any_neg);
        if (any_neg) atomicOr(flag, XF_NEGATIVE);
        finish_moments(t, chk, flag, true);
    }
}

// Covered coarse cells: restriction of the fine state, stress rescaled
// fine -> coarse.  blockIdx.y == 0: the three-cell ring of the box outside
// its core, 32 coarse cells per block; warp w reads child w (x, y, z bits of
// w), warp 0 averages the eight children and prepares the fields, every warp
// writes its own directions.  blockIdx.y == 1: core cells take the free stream.
template <typename Sc, typename Sf>
__global__ void __launch_bounds__(SPLIT_THREADS, 2)
    k_restrict(Sc *__restrict__ coarse, Grid G, const Sf *__restrict__ fine, Grid F, BoxSpec B, int pad,
               const double *__restrict__ free_g, Rescale r, int *__restrict__ flag) {
    chain_wait();
    using T = typename Store<Sc>::A;
    __shared__ SplitShared<T> sh;
    if (blockIdx.y == 1) {
        // the covered core takes the free-stream populations: converted to
        // the storage form once per block (as store_g converts them), then
        // copied to every core cell
        __shared__ Sc free_s[Q];
        const int cx0 = B.bx - 6, cy0 = B.by - 6;
        if (cx0 <= 0 || cy0 <= 0) return;
        if (threadIdx.x < Q)
            Store<Sc>::store(&free_s[threadIdx.x], threadIdx.x, (typename Store<Sc>::T)free_g[threadIdx.x],
                             G.shift[threadIdx.x]);
        __syncthreads();
        const long long ncore = (long long)cx0 * cy0 * B.bz;
        const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= ncore) return;
        const int x = (int)(i % cx0);
        const long long rest = i / cx0;
        const int y = (int)(rest % cy0), z = (int)(rest / cy0);
        Sc *const cell = coarse + G.cell(B.lo[0] + 3 + x + 1, B.lo[1] + 3 + y + 1, B.lo[2] + z);
#pragma unroll
        for (int q = 0; q < Q; ++q) cell[q * G.qs] = free_s[q];
        return;
    }
    const long long nring = ring_count(B.bx, B.by, 3, 3), n = nring * B.bz;
    if ((long long)blockIdx.x * SPLIT_CELLS >= n) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const long long i = (long long)blockIdx.x * SPLIT_CELLS + lane;
    const bool valid = i < n;
    int bx = 0, by = 0, z = 0;
    if (valid) {
        z = (int)(i / nring);
        ring_cell(i - z * nring, B.bx, B.by, 3, 3, bx, by);
    }
    const int fx = pad + 2 * bx + (w & 1), fy = pad + 2 * by + ((w >> 1) & 1), fz = 2 * z + (w >> 2);
    T v[Q], s[10];
    bool neg = false;
    static_for<0, Q>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        v[q] = valid ? load_as<T>(fine, F, q, fx + 1, fy + 1, fz) : T(0);
        neg |= v[q] < T(-weight(q));
    });
    cell_moments(v, s);
    T mc[10];
    finish_moments(s, mc, flag, valid);
    put_partial(sh, mc, neg);
    __syncthreads();
    if (w == 0) {
        T m[10];
        bool any_neg;
        sum_partials(sh, m, any_neg);
        if (valid && any_neg) atomicOr(flag, XF_NEGATIVE);
#pragma unroll
        for (int k = 0; k < 10; ++k) m[k] *= T(0.125);
        rescale_stress(m, r);
        if (valid) check_fields(m, flag);
        put_fields(sh, 0, m);
    }
    __syncthreads();
    T m[10], fac[9];
    get_fields(sh, 0, m, fac);
    const int cxi = B.lo[0] + bx, cyi = B.lo[1] + by, czi = B.lo[2] + z;
    bool bad = false;
    by_warp([&](auto wc) {
        owned<decltype(wc)::value>([&](auto qc, int) {
            constexpr int q = decltype(qc)::value;
            const T g = population<q>(m, fac, bad);
            if (valid) store_as<T>(coarse, G, q, cxi + 1, cyi + 1, czi, g);
        });
    });
    if (bad && valid) atomicOr(flag, XF_NEGATIVE);
}

// ------------------------------------------------------------ budgets and validity
// Inflow of mass and momentum through the outer x and y faces of the coarse
// lattice, from the state the streaming reads (refined_solver.py:215-222,
// 274-278): partials[face][block][4] hold the block sums of the face flux.
// The z pair of faces is left out: with z periodic its two fluxes are equal.
template <typename S>
__global__ void __launch_bounds__(256)
    k_outer_flux(const S *__restrict__ pdf, Grid G, const FluxTerm *__restrict__ terms0,
                 const FluxTerm *__restrict__ terms1, int nterms, const Face *__restrict__ faces, int nfaces,
                 double *__restrict__ partials) {
    const int f = blockIdx.y;
    if (f >= nfaces) return;
    const Face F = faces[f];
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double acc[4] = {0, 0, 0, 0};
    if (i < (long long)F.n1 * F.n2) {
        const int t1 = (int)(i / F.n2), t2 = (int)(i - (long long)t1 * F.n2);
        const FluxTerm *terms = F.axis == 0 ? terms0 : terms1;
        for (int t = 0; t < nterms; ++t)
            face_term_add(pdf, G, terms[t], F.axis, F.coarse_index, F.lo1 + t1, F.lo2 + t2, false, acc);
    }
    block_sum_store<4>(acc, partials + (long long)f * 4 * gridDim.x);
}

// out[k] = sum over faces (in order) of -side * dx^3 * sum over blocks, for
// this step; out[4 + k] accumulates it over the tracked steps
__global__ void __launch_bounds__(REDUCE_THREADS)
    k_outer_final(const double *__restrict__ partials, const Face *__restrict__ faces, int nfaces, int nblocks,
                  double volume, double *__restrict__ out) {
    double total[4] = {0, 0, 0, 0};
    for (int f = 0; f < nfaces; ++f) {
        double s[4];
        reduce_rows<4>(partials + (long long)f * nblocks * 4, nblocks, 0u, s);
        for (int k = 0; k < 4; ++k) total[k] -= faces[f].side * s[k] * volume;
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 4; ++k) {
            out[k] = total[k];
            out[4 + k] += total[k];
        }
}


// Statistics of one level's region (refined_solver.py:291-299, 347-361):
// fluid cells of [x0, x1) x [y0, y1) x all z (interior coordinates) outside
// [ex0, ex1) x [ey0, ey1).  partials[block][NSTAT] = max |u|^2, max |rho - 1|,
// sum drho, sum j (3), cells, non-finite cells.
struct Region {
    int x0, x1, y0, y1, ex0, ex1, ey0, ey1;
};

// drho = sum g and j = sum c g of one cell, summed along the z lines first
// (51 FP64 additions instead of 80)
template <typename S>
__device__ __forceinline__ void mass_momentum(const S *__restrict__ cell, const Grid &G, double &drho, double j[3]) {
    double col[3][3], jz = 0.0;
#pragma unroll
    for (int ix = 0; ix < 3; ++ix)
#pragma unroll
        for (int iy = 0; iy < 3; ++iy) {
            const int qa = qof(ix, iy, 0), qb = qof(ix, iy, 1), qc = qof(ix, iy, 2);
            const double a = (double)Store<S>::load(cell + qa * G.qs, qa, G.shift[qa]);
            const double b = (double)Store<S>::load(cell + qb * G.qs, qb, G.shift[qb]);
            const double c = (double)Store<S>::load(cell + qc * G.qs, qc, G.shift[qc]);
            col[ix][iy] = (a + c) + b;
            jz += c - a;
        }
    double sx[3], sy[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        sx[k] = (col[k][0] + col[k][1]) + col[k][2];
        sy[k] = (col[0][k] + col[1][k]) + col[2][k];
    }
    drho = (sx[0] + sx[1]) + sx[2];
    j[0] = sx[2] - sx[0];
    j[1] = sy[2] - sy[0];
    j[2] = jz;
}
constexpr int NSTAT = CELL_STATS;
template <typename S>
__global__ void __launch_bounds__(256)
    k_region_stats(const S *__restrict__ pdf, Grid G, const uint8_t *__restrict__ flags, Region R,
                   double *__restrict__ partials) {
    const int w = R.x1 - R.x0, h = R.y1 - R.y0;
    const long long nrows = (long long)h * G.nz;
    double a[NSTAT] = {0, 0, 0, 0, 0, 0, 0, 0};
    // blocks walk the region's (y, z) rows, threads its x
    for (long long row = blockIdx.x; row < nrows; row += gridDim.x)
    for (int xx = threadIdx.x; xx < w; xx += blockDim.x) {
        const int z = (int)(row / h), y = R.y0 + (int)(row - (long long)z * h), x = R.x0 + xx;
        if (x >= R.ex0 && x < R.ex1 && y >= R.ey0 && y < R.ey1) continue;
        if (flags[(y + 1) * G.nxp + (x + 1)] != FLAG_FLUID) continue;
        double drho, j[3];
        mass_momentum(pdf + G.cell(x + 1, y + 1, z), G, drho, j);
        const double rho = drho + 1.0, inv = 1.0 / rho;
        const double u[3] = {j[0] * inv, j[1] * inv, j[2] * inv};
        const double u2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
        if (!isfinite(rho) || !isfinite(u2)) {
            a[7] += 1.0;
            continue;
        }
        a[0] = fmax(a[0], u2);
        a[1] = fmax(a[1], fabs(rho - 1.0));
        a[2] += drho;
        a[3] += j[0];
        a[4] += j[1];
        a[5] += j[2];
        a[6] += 1.0;
    }
    __shared__ double red[8][NSTAT];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        a[0] = fmax(a[0], __shfl_down_sync(0xffffffffu, a[0], o));
        a[1] = fmax(a[1], __shfl_down_sync(0xffffffffu, a[1], o));
        for (int k = 2; k < NSTAT; ++k) a[k] += __shfl_down_sync(0xffffffffu, a[k], o);
    }
    if (lane == 0)
        for (int k = 0; k < NSTAT; ++k) red[warp][k] = a[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = blockDim.x >> 5;
        for (int wv = 1; wv < nw; ++wv) {
            red[0][0] = fmax(red[0][0], red[wv][0]);
            red[0][1] = fmax(red[0][1], red[wv][1]);
            for (int k = 2; k < NSTAT; ++k) red[0][k] += red[wv][k];
        }
        for (int k = 0; k < NSTAT; ++k) partials[(long long)blockIdx.x * NSTAT + k] = red[0][k];
    }
}

// The budget's sums over the same region on the integer pipe: each fluid
// cell's drho and j from its 27 populations as fixed point (FIX_BITS), one
// cell per thread (the kernel is bound by load latency: a thread looping
// over four cells took four times as long), one row per warp (CELL_STATS
// layout, maxima left 0).  A population of magnitude 1 or more (no valid
// zero-centred population has one) or a non-finite one makes the cell
// invalid; with that bound a row of 32 cells stays inside 64 bits.  rows:
// region_sum_rows(cells) of them.
constexpr int SUM_CELLS_PER_THREAD = 1;
__host__ __device__ constexpr long long region_sum_rows(long long cells) {
    return (cells + 256 * SUM_CELLS_PER_THREAD - 1) / (256 * SUM_CELLS_PER_THREAD) * 8;
}
template <typename S>
__global__ void __launch_bounds__(256)
    k_region_sums(const S *__restrict__ pdf, Grid G, const uint8_t *__restrict__ flags, Region R,
                  long long *__restrict__ rows) {
    chain_wait();
    const int w = R.x1 - R.x0, h = R.y1 - R.y0;
    const long long n = (long long)w * h * G.nz;
    BudgetSums acc;
#pragma unroll 1
    for (int k = 0; k < SUM_CELLS_PER_THREAD; ++k) {
        const long long i = ((long long)blockIdx.x * SUM_CELLS_PER_THREAD + k) * 256 + threadIdx.x;
        if (i >= n) break;
        const int z = (int)(i / ((long long)w * h));
        const int r = (int)(i - (long long)z * w * h);
        const int y = R.y0 + r / w, x = R.x0 + r % w;
        if (x >= R.ex0 && x < R.ex1 && y >= R.ey0 && y < R.ey1) continue;
        if (flags[(y + 1) * G.nxp + (x + 1)] != FLAG_FLUID) continue;
        const S *cell = pdf + G.cell(x + 1, y + 1, z);
        long long f[Q];
        bool ok = true;
#pragma unroll
        for (int q = 0; q < Q; ++q) ok &= fixed_of<0>(Store<S>::load(cell + q * G.qs, q, G.shift[q]), f[q]);
        if (!ok) {
            ++acc.bad;
            continue;
        }
        // sums along z first, as mass_momentum does (exact in integers)
        long long col[3][3], jz = 0;
#pragma unroll
        for (int ix = 0; ix < 3; ++ix)
#pragma unroll
            for (int iy = 0; iy < 3; ++iy) {
                const long long a = f[qof(ix, iy, 0)], b = f[qof(ix, iy, 1)], c = f[qof(ix, iy, 2)];
                col[ix][iy] = a + b + c;
                jz += c - a;
            }
        long long sx[3], sy[3];
#pragma unroll
        for (int k2 = 0; k2 < 3; ++k2) {
            sx[k2] = col[k2][0] + col[k2][1] + col[k2][2];
            sy[k2] = col[0][k2] + col[1][k2] + col[2][k2];
        }
        acc.drho += sx[0] + sx[1] + sx[2];
        acc.jx += sx[2] - sx[0];
        acc.jy += sy[2] - sy[0];
        acc.jz += jz;
        ++acc.cells;
    }
    warp_budget_row(acc, rows, (long long)blockIdx.x * 8 + (threadIdx.x >> 5));
}

// first stage of a reduction of many statistics rows: block b reduces rows
// [b REDUCE_THREADS, (b + 1) REDUCE_THREADS) into out[b], so that the final
// block reduces one row per stage block (a fixed order either way)
__global__ void __launch_bounds__(REDUCE_THREADS)
    k_region_stage(const double *__restrict__ partials, long long nrows, double *__restrict__ out) {
    const long long first = (long long)blockIdx.x * REDUCE_THREADS;
    double a[NSTAT];
    reduce_rows<NSTAT>(partials + first * NSTAT, min((long long)REDUCE_THREADS, nrows - first), 0x3u, a);
    if (threadIdx.x == 0)
        for (int k = 0; k < NSTAT; ++k) out[(long long)blockIdx.x * NSTAT + k] = a[k];
}

__global__ void __launch_bounds__(REDUCE_THREADS)
    k_region_final(const double *__restrict__ partials, int nblocks, double *__restrict__ out) {
    double a[NSTAT];
    reduce_rows<NSTAT>(partials, nblocks, 0x3u, a);
    if (threadIdx.x == 0)
        for (int k = 0; k < NSTAT; ++k) out[k] = a[k];
}

// The budget's integer rows (warp_budget_row) into the CELL_STATS doubles:
// each row converted once, then the fixed-order reduction of k_region_stage
// (block b: rows [b REDUCE_THREADS, (b + 1) REDUCE_THREADS), one row each)
// or of k_region_final (one block, every row)
__global__ void __launch_bounds__(REDUCE_THREADS)
    k_budget_stage(const long long *__restrict__ rows, long long nrows, double *__restrict__ out,
                   unsigned *__restrict__ done = nullptr, double *__restrict__ total = nullptr) {
    const long long b = (long long)blockIdx.x * REDUCE_THREADS + threadIdx.x;
    double a[NSTAT] = {-INFINITY, -INFINITY, 0, 0, 0, 0, 0, 0};
    if (b < nrows) budget_row_values(rows + b * NSTAT, a);
    reduce_block<NSTAT>(0x3u, a);
    if (threadIdx.x == 0)
        for (int k = 0; k < NSTAT; ++k) out[(long long)blockIdx.x * NSTAT + k] = a[k];
    if (!done) return;
    // done: the last block to finish reduces the stage rows into total[NSTAT]
    // in k_region_final's order (same result), and leaves done at 0
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(done, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
#pragma unroll
    for (int k = 0; k < NSTAT; ++k) a[k] = k < 2 ? -INFINITY : 0.0;
    for (long long r = threadIdx.x; r < (long long)gridDim.x; r += REDUCE_THREADS)
#pragma unroll
        for (int k = 0; k < NSTAT; ++k) {
            const double v = __ldcg(out + r * NSTAT + k);
            a[k] = k < 2 ? fmax(a[k], v) : a[k] + v;
        }
    reduce_block<NSTAT>(0x3u, a);
    if (threadIdx.x == 0) {
        for (int k = 0; k < NSTAT; ++k) total[k] = a[k];
        *done = 0;
    }
}
__global__ void __launch_bounds__(REDUCE_THREADS)
    k_budget_final(const long long *__restrict__ rows, long long nrows, double *__restrict__ out) {
    double a[NSTAT] = {-INFINITY, -INFINITY, 0, 0, 0, 0, 0, 0};
    for (long long b = threadIdx.x; b < nrows; b += REDUCE_THREADS) {
        double v[NSTAT];
        budget_row_values(rows + b * NSTAT, v);
        a[0] = fmax(a[0], v[0]);
        a[1] = fmax(a[1], v[1]);
#pragma unroll
        for (int k = 2; k < NSTAT; ++k) a[k] += v[k];
    }
    reduce_block<NSTAT>(0x3u, a);
    if (threadIdx.x == 0)
        for (int k = 0; k < NSTAT; ++k) out[k] = a[k];
}

// ------------------------------------------------------------ stationarity residuals
// d(rho, j / U)/dt over a region's fluid cells (convergence.py:58-96) against
// a snapshot kept on the device: partials[block][9] = sum of squares (4),
// max |.| (4), cells; the snapshot takes the current values.  With reset the
// snapshot is only taken.
template <typename S>
__global__ void __launch_bounds__(256)
    k_residuals(const S *__restrict__ pdf, Grid G, const uint8_t *__restrict__ flags, Region R,
                double *__restrict__ snapshot, double inv_speed, double inv_dt, int reset,
                double *__restrict__ partials) {
    const int w = R.x1 - R.x0, h = R.y1 - R.y0;
    const long long nrows = (long long)h * G.nz;
    double sq[4] = {0, 0, 0, 0}, mx[4] = {0, 0, 0, 0}, cells = 0.0;
    // blocks walk the region's (y, z) rows, threads its x; the snapshot is
    // indexed by the cell's place in the region, (z h + y - y0) w + x - x0
    for (long long row = blockIdx.x; row < nrows; row += gridDim.x)
    for (int xx = threadIdx.x; xx < w; xx += blockDim.x) {
        const int z = (int)(row / h), y = R.y0 + (int)(row - (long long)z * h), x = R.x0 + xx;
        const long long i = row * w + xx;
        if (x >= R.ex0 && x < R.ex1 && y >= R.ey0 && y < R.ey1) continue;
        if (flags[(y + 1) * G.nxp + (x + 1)] != FLAG_FLUID) continue;
        double drho, j[3];
        mass_momentum(pdf + G.cell(x + 1, y + 1, z), G, drho, j);
        const double cur[4] = {drho + 1.0, j[0] * inv_speed, j[1] * inv_speed, j[2] * inv_speed};
        double *s = snapshot + 4 * i;
        if (!reset) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const double d = (cur[k] - s[k]) * inv_dt;
                sq[k] += d * d;
                mx[k] = fmax(mx[k], fabs(d));
            }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) s[k] = cur[k];
        cells += 1.0;
    }
    __shared__ double red[8][9];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        for (int k = 0; k < 4; ++k) {
            sq[k] += __shfl_down_sync(0xffffffffu, sq[k], o);
            mx[k] = fmax(mx[k], __shfl_down_sync(0xffffffffu, mx[k], o));
        }
        cells += __shfl_down_sync(0xffffffffu, cells, o);
    }
    if (lane == 0) {
        for (int k = 0; k < 4; ++k) {
            red[warp][k] = sq[k];
            red[warp][4 + k] = mx[k];
        }
        red[warp][8] = cells;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int wv = 1; wv < (int)(blockDim.x >> 5); ++wv) {
            for (int k = 0; k < 4; ++k) {
                red[0][k] += red[wv][k];
                red[0][4 + k] = fmax(red[0][4 + k], red[wv][4 + k]);
            }
            red[0][8] += red[wv][8];
        }
        for (int k = 0; k < 9; ++k) partials[(long long)blockIdx.x * 9 + k] = red[0][k];
    }
}

__global__ void __launch_bounds__(REDUCE_THREADS)
    k_residuals_final(const double *__restrict__ partials, int nblocks, double *__restrict__ out) {
    double a[9];
    reduce_rows<9>(partials, nblocks, 0xF0u, a);
    if (threadIdx.x == 0)
        for (int k = 0; k < 9; ++k) out[k] = a[k];
}

}  // namespace ak
