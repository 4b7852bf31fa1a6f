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
#include "ak_kernels.cuh"

namespace ak {

constexpr double TCS2 = 1.0 / 3.0;
// second-order index pairs (xx, yy, zz, xy, xz, yz)
__host__ __device__ constexpr int sa(int k) { return k < 3 ? k : (k == 5 ? 1 : 0); }
__host__ __device__ constexpr int sb(int k) { return k < 3 ? k : (k == 3 ? 1 : 2); }

// error flags of the transfer checks
constexpr int XF_DENSITY = 1, XF_NEGATIVE = 2, XF_MACH = 4, XF_NONFINITE = 8;

__device__ __forceinline__ void transfer_moments(const double g[Q], double m[10], int *flag) {
    double drho = 0.0, j[3] = {0, 0, 0}, pi[6] = {0, 0, 0, 0, 0, 0};
    bool negative = false;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const double v = g[q];
        const int c[3] = {cx(q), cy(q), cz(q)};
        drho += v;
        j[0] += c[0] * v;
        j[1] += c[1] * v;
        j[2] += c[2] * v;
#pragma unroll
        for (int k = 0; k < 6; ++k) pi[k] += (double)(c[sa(k)] * c[sb(k)]) * v;
        negative |= v + weight(q) < 0.0;
    }
    const double rho = drho + 1.0;
    if (!(rho > 0.0)) atomicOr(flag, XF_DENSITY);
    if (negative) atomicOr(flag, XF_NEGATIVE);
    if (sqrt(j[0] * j[0] + j[1] * j[1] + j[2] * j[2]) / rho / sqrt(TCS2) > 0.3) atomicOr(flag, XF_MACH);
    m[0] = rho;
    m[1] = j[0];
    m[2] = j[1];
    m[3] = j[2];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        double p = pi[k];
        if (k < 3) p -= drho * TCS2;
        m[4 + k] = p - j[sa(k)] * j[sb(k)] / rho;
    }
}

// zero-centred populations from (rho, j, Pi_neq), refinement.py:177-203
__device__ __forceinline__ void transfer_populations(const double m[10], double g[Q], int *flag) {
    const double rho = m[0];
    if (!(rho > 0.0)) atomicOr(flag, XF_DENSITY);
    if (sqrt(m[1] * m[1] + m[2] * m[2] + m[3] * m[3]) / rho / sqrt(TCS2) > 0.3) atomicOr(flag, XF_MACH);
    const double u[3] = {m[1] / rho, m[2] / rho, m[3] / rho};
    bool bad = false;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int c[3] = {cx(q), cy(q), cz(q)};
        double eq = 1.0;
#pragma unroll
        for (int a = 0; a < 3; ++a)
            eq *= c[a] == 0 ? 2.0 / 3.0 - u[a] * u[a] : (TCS2 + u[a] * u[a] + c[a] * u[a]) / 2.0;
        eq *= rho;
        double neq = 0.0;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            double h = (double)(c[sa(k)] * c[sb(k)]) - (k < 3 ? TCS2 : 0.0);
            if (k >= 3) h *= 2.0;
            neq += weight(q) * h / (2.0 * TCS2 * TCS2) * m[4 + k];
        }
        const double f = eq + neq;
        bad |= !isfinite(f) || f < 0.0;
        g[q] = f - weight(q);
    }
    if (bad) atomicOr(flag, XF_NEGATIVE);
}

struct Rescale {
    double shear, bulk;  // target tau dt / source tau dt
};
__device__ __forceinline__ void rescale_stress(double m[10], Rescale r) {
    const double iso = (m[4] + m[5] + m[6]) / 3.0;
#pragma unroll
    for (int k = 4; k < 10; ++k) m[k] *= r.shear;
#pragma unroll
    for (int k = 4; k < 7; ++k) m[k] += (r.bulk - r.shear) * iso;
}

// ------------------------------------------------------------ split step
template <typename S>
__global__ void __launch_bounds__(128, Store<S>::MIN_BLOCKS)
    k_collide(S *__restrict__ pdf, const uint8_t *__restrict__ flags, Grid G, Shift27 shift,
              typename Store<S>::T omega_s, typename Store<S>::T omega_b) {
    using T = typename Store<S>::T;
    const int x = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int y = blockIdx.y + 1;
    const int z = blockIdx.z;
    if (x > G.nx) return;
    if (__ldg(flags + y * G.nxp + x) != FLAG_FLUID) return;
    const long long c = G.cell(x, y, z);
    T g[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) g[q] = Store<S>::load(pdf + q * G.qs + c, q, shift.v[q]);
    if constexpr (sizeof(T) == 8)
        collide_full<T>(g, T(1) - omega_s, omega_b);
    else
        collide<T>(g, omega_s, omega_b);
#pragma unroll
    for (int q = 0; q < Q; ++q) Store<S>::store(pdf + q * G.qs + c, q, g[q], shift.v[q]);
}

// pull streaming of the stored values (bit copies); x and y wrap when periodic
template <typename S>
__global__ void k_stream(const S *__restrict__ src, S *__restrict__ dst, const uint8_t *__restrict__ flags, Grid G,
                         int periodic_xy) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int y = blockIdx.y + 1;
    const int z = blockIdx.z;
    if (x > G.nx) return;
    if (__ldg(flags + y * G.nxp + x) != FLAG_FLUID) return;
    const long long c = G.cell(x, y, z);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        int xs = x - cx(q), ys = y - cy(q);
        if (periodic_xy) {
            xs = xs < 1 ? xs + G.nx : (xs > G.nx ? xs - G.nx : xs);
            ys = ys < 1 ? ys + G.ny : (ys > G.ny ? ys - G.ny : ys);
        }
        dst[q * G.qs + c] = src[q * G.qs + G.cell(xs, ys, G.wrapz(z - cz(q)))];
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

// flux of one face patch entry (t1, t2) at lattice coordinates; periodic wraps
// every axis (interior coordinates)
template <typename S>
__device__ void face_flux_entry(const S *pdf, const Grid &G, const FluxTerm *terms, int nterms, int axis, int index,
                                int p1, int p2, bool periodic, double out[4]) {
    const int a1 = axis == 0 ? 1 : 0, a2 = axis == 2 ? 1 : 2;
    const int dims[3] = {G.nx, G.ny, G.nz};
    for (int k = 0; k < 4; ++k) out[k] = 0.0;
    for (int t = 0; t < nterms; ++t) {
        const FluxTerm T = terms[t];
        const int normal = axis == 0 ? cx(T.d) : (axis == 1 ? cy(T.d) : cz(T.d));
        int c3[3];
        c3[axis] = index + (normal < 0 ? 1 : 0);
        c3[a1] = p1 + T.shift[a1];
        c3[a2] = p2 + T.shift[a2];
        if (periodic)
            for (int a = 0; a < 3; ++a) c3[a] = (c3[a] % dims[a] + dims[a]) % dims[a];
        else
            c3[2] = (c3[2] % dims[2] + dims[2]) % dims[2];
        const double v = load_g(pdf, G, T.d, c3[0] + 1, c3[1] + 1, c3[2]);
        for (int k = 0; k < 4; ++k) out[k] += v * T.coef[k];
    }
}

// coarse faces: reg[face][t1][t2][4] = flux * dx^3
template <typename S>
__global__ void k_face_flux_coarse(const S *__restrict__ pdf, Grid G, const FluxTerm *__restrict__ terms0,
                                   const FluxTerm *__restrict__ terms1, int nterms, const Face *__restrict__ faces,
                                   int nfaces, const long long *__restrict__ offsets, double scale,
                                   double *__restrict__ reg) {
    const int f = blockIdx.y;
    if (f >= nfaces) return;
    const Face F = faces[f];
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)F.n1 * F.n2) return;
    const int t1 = (int)(i / F.n2), t2 = (int)(i - (long long)t1 * F.n2);
    double out[4];
    face_flux_entry(pdf, G, F.axis == 0 ? terms0 : terms1, nterms, F.axis, F.coarse_index, F.lo1 + t1, F.lo2 + t2,
                    true, out);
    double *r = reg + offsets[f] + 4 * i;
    for (int k = 0; k < 4; ++k) r[k] = out[k] * scale;
}

// fine faces: each coarse entry accumulates the sum of its 2 x 2 fine entries
template <typename S>
__global__ void k_face_flux_fine(const S *__restrict__ pdf, Grid G, const FluxTerm *__restrict__ terms0,
                                 const FluxTerm *__restrict__ terms1, int nterms, const Face *__restrict__ faces,
                                 int nfaces, const long long *__restrict__ offsets, int pad, double scale,
                                 double *__restrict__ reg) {
    const int f = blockIdx.y;
    if (f >= nfaces) return;
    const Face F = faces[f];
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)F.n1 * F.n2) return;
    const int t1 = (int)(i / F.n2), t2 = (int)(i - (long long)t1 * F.n2);
    // fine tangential origin: x and y start after the donor padding, z at 0
    const int a1 = F.axis == 0 ? 1 : 0, a2 = F.axis == 2 ? 1 : 2;
    const int o1 = a1 < 2 ? pad : 0, o2 = a2 < 2 ? pad : 0;
    double sum[4] = {0, 0, 0, 0};
    for (int s1 = 0; s1 < 2; ++s1)
        for (int s2 = 0; s2 < 2; ++s2) {
            double out[4];
            face_flux_entry(pdf, G, F.axis == 0 ? terms0 : terms1, nterms, F.axis, F.fine_index,
                            o1 + 2 * t1 + s1, o2 + 2 * t2 + s2, false, out);
            for (int k = 0; k < 4; ++k) sum[k] += out[k];
        }
    double *r = reg + offsets[f] + 4 * i;
    for (int k = 0; k < 4; ++k) r[k] += sum[k] * scale;
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

// moments of the donor block: coarse cells [lo-3, hi+3) in x and y (periodic
// wrap, as the reference indexes them), all z; covered core cells take the
// free-stream populations
template <typename S>
__global__ void k_block_moments(const S *__restrict__ pdf, Grid G, BoxSpec B, const double *__restrict__ free_g,
                                double *__restrict__ out, int *__restrict__ flag) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)B.dnx * B.dny * G.nz;
    if (i >= n) return;
    const int z = (int)(i % G.nz);
    const long long xy = i / G.nz;
    const int by = (int)(xy % B.dny), bx = (int)(xy / B.dny);
    int cxi = B.dx0 + bx, cyi = B.dy0 + by;
    cxi = (cxi % G.nx + G.nx) % G.nx;
    cyi = (cyi % G.ny + G.ny) % G.ny;
    double g[Q];
    if (in_core(B, cxi, cyi)) {
        for (int q = 0; q < Q; ++q) g[q] = free_g[q];
    } else {
        for (int q = 0; q < Q; ++q) g[q] = load_g(pdf, G, q, cxi + 1, cyi + 1, z);
    }
    double m[10];
    transfer_moments(g, m, flag);
    for (int k = 0; k < 10; ++k) out[i * 10 + k] = m[k];
}

// donor populations for the padding band of the fine block: prolongation of
// the time-interpolated donor moments, stress rescaled coarse -> fine
template <typename S>
__global__ void k_donors(S *__restrict__ fine, Grid F, BoxSpec B, int nzc, const double *__restrict__ mold,
                         const double *__restrict__ mnew, double fraction, Rescale r, int pad, int *__restrict__ flag) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)F.nx * F.ny * F.nz;
    if (i >= n) return;
    const int fz = (int)(i % F.nz);
    const long long xy = i / F.nz;
    const int fy = (int)(xy % F.ny), fx = (int)(xy / F.ny);  // 0-based padded coordinates
    const bool band = fx < pad || fx >= F.nx - pad || fy < pad || fy >= F.ny - pad;
    if (!band) return;
    // parent coarse cell relative to the donor block, and child side
    const int px = (fx >> 1) + 2, py = (fy >> 1) + 2, pz = fz >> 1;  // block x = lo-3 + px
    const double sgn[3] = {(fx & 1) ? 1.0 : -1.0, (fy & 1) ? 1.0 : -1.0, (fz & 1) ? 1.0 : -1.0};
    double wts[3][5];
    for (int a = 0; a < 3; ++a) {
        wts[a][0] = sgn[a] * (3.0 / 128.0);
        wts[a][1] = -sgn[a] * (11.0 / 64.0);
        wts[a][2] = 1.0;
        wts[a][3] = sgn[a] * (11.0 / 64.0);
        wts[a][4] = -sgn[a] * (3.0 / 128.0);
    }
    double m[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int kz = 0; kz < 5; ++kz) {
        const int zz = ((pz + kz - 2) % nzc + nzc) % nzc;
        for (int ky = 0; ky < 5; ++ky) {
            const int yy = py + ky - 2;
            for (int kx = 0; kx < 5; ++kx) {
                const int xx = px + kx - 2;
                const double w = wts[0][kx] * wts[1][ky] * wts[2][kz];
                const long long j = ((long long)xx * B.dny + yy) * nzc + zz;
                for (int k = 0; k < 10; ++k)
                    m[k] += w * ((1.0 - fraction) * mold[j * 10 + k] + fraction * mnew[j * 10 + k]);
            }
        }
    }
    rescale_stress(m, r);
    double g[Q];
    transfer_populations(m, g, flag);
    for (int q = 0; q < Q; ++q) store_g(fine, F, q, fx + 1, fy + 1, fz, g[q]);
}

// ------------------------------------------------------------ reflux, restriction
// coarse cells just outside each face: equilibrium part of the state shifted
// by the flux mismatch (interface.py:285-295)
template <typename S>
__global__ void k_reflux(S *__restrict__ pdf, Grid G, const Face *__restrict__ faces, int nfaces,
                         const long long *__restrict__ offsets, const double *__restrict__ reg_c,
                         const double *__restrict__ reg_f, double inv_volume, int *__restrict__ flag) {
    const int f = blockIdx.y;
    if (f >= nfaces) return;
    const Face F = faces[f];
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)F.n1 * F.n2) return;
    const int t1 = (int)(i / F.n2), t2 = (int)(i - (long long)t1 * F.n2);
    const int a1 = F.axis == 0 ? 1 : 0, a2 = F.axis == 2 ? 1 : 2;
    int c3[3];
    c3[F.axis] = F.side < 0 ? F.coarse_index : F.coarse_index + 1;  // the cell outside the box
    c3[a1] = F.lo1 + t1;
    c3[a2] = F.lo2 + t2;
    const double *rc = reg_c + offsets[f] + 4 * i, *rf = reg_f + offsets[f] + 4 * i;
    double g[Q], m_old[10], m_new[10], p_old[Q], p_new[Q];
    for (int q = 0; q < Q; ++q) g[q] = load_g(pdf, G, q, c3[0] + 1, c3[1] + 1, c3[2]);
    transfer_moments(g, m_old, flag);
    for (int k = 4; k < 10; ++k) m_old[k] = 0.0;
    for (int k = 0; k < 10; ++k) m_new[k] = m_old[k];
    for (int k = 0; k < 4; ++k) m_new[k] += F.side * (rf[k] - rc[k]) * inv_volume;
    transfer_populations(m_new, p_new, flag);
    transfer_populations(m_old, p_old, flag);
    for (int q = 0; q < Q; ++q) g[q] += p_new[q] - p_old[q];
    double chk[10];
    transfer_moments(g, chk, flag);
    for (int q = 0; q < Q; ++q) store_g(pdf, G, q, c3[0] + 1, c3[1] + 1, c3[2], g[q]);
}

// covered coarse cells: restriction of the fine state (core cells take the
// free stream), stress rescaled fine -> coarse
template <typename Sc, typename Sf>
__global__ void k_restrict(Sc *__restrict__ coarse, Grid G, const Sf *__restrict__ fine, Grid F, BoxSpec B, int pad,
                           const double *__restrict__ free_g, Rescale r, int *__restrict__ flag) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)B.bx * B.by * B.bz;
    if (i >= n) return;
    const int z = (int)(i % B.bz);
    const long long xy = i / B.bz;
    const int by = (int)(xy % B.by), bx = (int)(xy / B.by);
    const int cxi = B.lo[0] + bx, cyi = B.lo[1] + by, czi = B.lo[2] + z;
    double g[Q];
    if (in_core(B, cxi, cyi)) {
        for (int q = 0; q < Q; ++q) g[q] = free_g[q];
    } else {
        double m[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int s = 0; s < 8; ++s) {
            const int fx = pad + 2 * bx + (s & 1), fy = pad + 2 * by + ((s >> 1) & 1), fz = 2 * z + (s >> 2);
            double gc[Q], mc[10];
            for (int q = 0; q < Q; ++q) gc[q] = load_g(fine, F, q, fx + 1, fy + 1, fz);
            transfer_moments(gc, mc, flag);
            for (int k = 0; k < 10; ++k) m[k] += mc[k];
        }
        for (int k = 0; k < 10; ++k) m[k] *= 0.125;
        rescale_stress(m, r);
        transfer_populations(m, g, flag);
    }
    for (int q = 0; q < Q; ++q) store_g(coarse, G, q, cxi + 1, cyi + 1, czi, g[q]);
}

}  // namespace ak
