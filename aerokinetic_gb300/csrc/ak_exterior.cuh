// ak_exterior.cuh -- the exterior_regularized_fd_v1 farfield (src/aerokinetic/
// exterior.py:18-200, wired in solver.py:36-41, 81-89, 179-201, 204-271).
//
// The physical lattice is padded by one auxiliary cell in x and y, the ring,
// which is exactly the ghost layer of the engine's padded layout.  The
// reference steps the padded lattice in collide-stream order and, after each
// stream, overwrites the ring with populations rebuilt from a predicted
// macroscopic state.  Here the case keeps post-collision populations, like
// the uniform solver, so the bulk stays one fused stream-collide pass; the
// ring work is a few small kernels over the ring and the two layers inside it:
//
//   band  (log rho, u) of every cell within two cells of the storage edge, for
//         the state the reference reads at the start of a step (its
//         pre-collision populations are the pull of the stored ones)
//   stage SSP-RK3 predictor of the ring state (exterior.py:81-151), one launch
//         per stage because each stage reads its ring neighbours' last stage
//   ring  the regularised populations of the predicted state (exterior.py:
//         153-171), the change they make to the streamed ones (the exterior
//         source, exterior.py:186-200), their macros for the next step, and
//         their collision into the next stored state
//
// All ring arithmetic is FP64 whatever the storage form: the ring holds about
// 2 (nx + ny) nz cells, a fraction of a percent of the lattice.
#pragma once
#include "ak_kernels.cuh"

namespace ak {

struct ExtGeom {
    int NX, NY;        // storage plane: the padded columns (nx + 2, ny + 2)
    int nz;
    int nring;         // ring cells per z plane
    int nband;         // cells within two cells of the edge, per z plane
    double speed;      // freestream (speed, 0, 0)
};

inline ExtGeom make_ext_geom(int nx, int ny, int nz, double speed) {
    ExtGeom E;
    E.NX = nx + 2;
    E.NY = ny + 2;
    E.nz = nz;
    E.nring = 2 * E.NX + 2 * (E.NY - 2);
    E.nband = 6 * E.NX + 6 * (E.NY - 6);
    E.speed = speed;
    return E;
}

// ring order: row y = 0, row y = NY - 1, column x = 0, column x = NX - 1
// (rows first, so most ring threads of a warp touch consecutive x)
__device__ __forceinline__ void ring_cell(const ExtGeom &E, int r, int &x, int &y) {
    if (r < E.NX) {
        x = r;
        y = 0;
    } else if (r < 2 * E.NX) {
        x = r - E.NX;
        y = E.NY - 1;
    } else if (r < 2 * E.NX + E.NY - 2) {
        x = 0;
        y = r - 2 * E.NX + 1;
    } else {
        x = E.NX - 1;
        y = r - 2 * E.NX - (E.NY - 2) + 1;
    }
}
__device__ __forceinline__ bool on_ring(const ExtGeom &E, int x, int y) {
    return x == 0 || y == 0 || x == E.NX - 1 || y == E.NY - 1;
}
__device__ __forceinline__ int ring_index(const ExtGeom &E, int x, int y) {
    if (y == 0) return x;
    if (y == E.NY - 1) return E.NX + x;
    if (x == 0) return 2 * E.NX + y - 1;
    return 2 * E.NX + E.NY - 2 + y - 1;
}
// band: rows 0..2 and NY-3..NY-1 in full, then columns 0..2 and NX-3..NX-1
__device__ __forceinline__ int band_index(const ExtGeom &E, int x, int y) {
    if (y < 3) return y * E.NX + x;
    if (y >= E.NY - 3) return (y - E.NY + 6) * E.NX + x;
    return 6 * E.NX + (y - 3) * 6 + (x < 3 ? x : x - E.NX + 6);
}
__device__ __forceinline__ void band_cell(const ExtGeom &E, int b, int &x, int &y) {
    if (b < 6 * E.NX) {
        const int row = b / E.NX;
        x = b - row * E.NX;
        y = row < 3 ? row : E.NY - 6 + row;
    } else {
        b -= 6 * E.NX;
        const int k = b % 6;
        y = 3 + b / 6;
        x = k < 3 ? k : E.NX - 6 + k;
    }
}

// (log rho, u) arrays laid out [component][z][cell]
struct ExtState {
    const double *ring;  // ring values of the current stage, or null: read the band
    const double *band;
};
__device__ __forceinline__ double ext_value(const ExtGeom &E, const ExtState &St, int x, int y, int z, int k) {
    if (St.ring && on_ring(E, x, y)) return St.ring[((long long)k * E.nz + z) * E.nring + ring_index(E, x, y)];
    return St.band[((long long)k * E.nz + z) * E.nband + band_index(E, x, y)];
}

struct RingPoint {
    int x, y, z, nvx, nvy;
    double n[3], ell, uninf, utinf[3];
};
__device__ __forceinline__ RingPoint ring_point(const ExtGeom &E, int x, int y, int z) {
    RingPoint p;
    p.x = x;
    p.y = y;
    p.z = z;
    p.nvx = x == 0 ? -1 : (x == E.NX - 1 ? 1 : 0);
    p.nvy = y == 0 ? -1 : (y == E.NY - 1 ? 1 : 0);
    p.ell = sqrt((double)(p.nvx * p.nvx + p.nvy * p.nvy));
    p.n[0] = p.nvx / p.ell;
    p.n[1] = p.nvy / p.ell;
    p.n[2] = 0.0;
    p.uninf = p.n[0] * E.speed;
    p.utinf[0] = E.speed - p.uninf * p.n[0];
    p.utinf[1] = -p.uninf * p.n[1];
    p.utinf[2] = -p.uninf * p.n[2];
    return p;
}

// d/dx_a of the four fields at a ring point along a non-periodic axis:
// second-order one-sided at the edge (edge -1 forward, +1 backward), central
// along the edge (exterior.py:69-79)
template <typename F>
__device__ __forceinline__ void edge_derivative(int edge, F &&at, double out[4]) {
    double c0, c1, c2;
    int o1, o2;
    if (edge == -1) {
        c0 = -1.5, c1 = 2.0, c2 = -0.5, o1 = 1, o2 = 2;
    } else if (edge == 1) {
        c0 = 1.5, c1 = -2.0, c2 = 0.5, o1 = -1, o2 = -2;
    } else {
        c0 = 0.0, c1 = -0.5, c2 = 0.5, o1 = -1, o2 = 1;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) out[k] = (c0 * at(0, k) + c1 * at(o1, k)) + c2 * at(o2, k);
}

// grad[a][k] = d field_k / d x_a at the ring point; z is periodic
__device__ __forceinline__ void ring_gradient(const ExtGeom &E, const ExtState &St, const RingPoint &p,
                                              double grad[3][4]) {
    edge_derivative(p.nvx, [&](int o, int k) { return ext_value(E, St, p.x + o, p.y, p.z, k); }, grad[0]);
    edge_derivative(p.nvy, [&](int o, int k) { return ext_value(E, St, p.x, p.y + o, p.z, k); }, grad[1]);
    const int zp = p.z + 1 == E.nz ? 0 : p.z + 1, zm = p.z == 0 ? E.nz - 1 : p.z - 1;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        grad[2][k] = (ext_value(E, St, p.x, p.y, zp, k) - ext_value(E, St, p.x, p.y, zm, k)) / 2;
}

// characteristic right-hand side of the ring state y (exterior.py:120-136)
__device__ __forceinline__ void ring_rhs(const ExtGeom &E, const ExtState &St, const RingPoint &p, const double y[4],
                                         double out[4]) {
    double grad[3][4];
    ring_gradient(E, St, p, grad);
    const double *n = p.n;
    double Gn[3], dq[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        dq[a] = grad[a][0];
        Gn[a] = grad[a][1] * n[0] + grad[a][2] * n[1] + grad[a][3] * n[2];
    }
    const double un = y[1] * n[0] + y[2] * n[1] + y[3] * n[2];
    const double rp = un + CS * y[0];
    double in[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) in[k] = ext_value(E, St, p.x - p.nvx, p.y - p.nvy, p.z, k);
    const double un_in = in[1] * n[0] + in[2] * n[1] + in[3] * n[2];
    const double rp_in = un_in + CS * in[0];
    const double div = ((grad[0][1] + grad[1][2]) + grad[2][3]) - (n[0] * Gn[0] + n[1] * Gn[1] + n[2] * Gn[2]);
    double sm = 0.0, sp = 0.0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        sm += p.utinf[a] * (Gn[a] - CS * dq[a]);
        sp += p.utinf[a] * (Gn[a] + CS * dq[a]);
    }
    const double r_minus = p.uninf * div - sm;
    const double r_plus = -(p.uninf + CS) * (rp - rp_in) / p.ell - sp - CS * div;
    double adv[3];
#pragma unroll
    for (int b = 0; b < 3; ++b) adv[b] = p.utinf[0] * grad[0][1 + b] + p.utinf[1] * grad[1][1 + b] +
                                         p.utinf[2] * grad[2][1 + b];
    const double adv_n = adv[0] * n[0] + adv[1] * n[1] + adv[2] * n[2];
    const double dq_n = dq[0] * n[0] + dq[1] * n[1] + dq[2] * n[2];
    out[0] = (r_plus - r_minus) / (2 * CS);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double tangent = y[1 + a] - un * n[a], tangent_in = in[1 + a] - un_in * n[a];
        const double d_t = -p.uninf * (tangent - tangent_in) / p.ell - (adv[a] - adv_n * n[a]) -
                           CS * CS * (dq[a] - dq_n * n[a]);
        out[1 + a] = n[a] * ((r_plus + r_minus) / 2) + d_t;
    }
}

// the initial state's u.n - cs log rho traced along the freestream to a
// glancing ring point (exterior.py:81-94): linear in x along the point's row,
// the freestream value (u_inf.n = 0) outside the storage
__device__ __forceinline__ double traced_incoming(const ExtGeom &E, const RingPoint &p, double time,
                                                  const double *__restrict__ inc0) {
    const double tx = p.x - E.speed * time;
    const double lo = floor(tx), f = tx - lo;
    const long long base = ((long long)(p.y == 0 ? 0 : 1) * E.nz + p.z) * E.NX;
    const int i0 = (int)lo, i1 = i0 + 1;
    const double v0 = (i0 >= 0 && i0 < E.NX) ? inc0[base + i0] : p.uninf;
    const double v1 = (i1 >= 0 && i1 < E.NX) ? inc0[base + i1] : p.uninf;
    return (1.0 - f) * v0 + f * v1;
}

// inflow and glancing points take the incoming invariant from outside
// (exterior.py:96-106)
__device__ __forceinline__ void ring_enforce(const ExtGeom &E, const RingPoint &p, double time,
                                             const double *__restrict__ inc0, double y[4]) {
    const bool inflow = p.uninf < 0, glancing = p.uninf == 0;
    if (!inflow && !glancing) return;
    const double *n = p.n;
    const double un = y[1] * n[0] + y[2] * n[1] + y[3] * n[2];
    const double rp = un + CS * y[0];
    const double rm = inflow ? p.uninf : traced_incoming(E, p, time, inc0);
    const double new_un = (rp + rm) / 2;
    y[0] = (rp - rm) / (2 * CS);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double tangent = inflow ? p.utinf[a] : y[1 + a] - un * n[a];
        y[1 + a] = new_un * n[a] + tangent;
    }
}

// ---------------------------------------------------------------- kernels
// (log rho, u) of the stored populations of every band cell (no pull): the
// initial state, before its first collision; also the initial incoming
// invariant of the two glancing rows
template <typename S>
__global__ void k_ext_band_direct(const S *__restrict__ pdf, Grid G, ExtGeom E, double *__restrict__ band,
                                  double *__restrict__ inc0) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)E.nband * E.nz) return;
    const int z = (int)(i / E.nband), b = (int)(i - (long long)z * E.nband);
    int x, y;
    band_cell(E, b, x, y);
    double rho, u[3];
    macro_at(pdf, G, x, y, z, rho, u);
    const double l = log(rho);
    const long long cs = (long long)E.nz * E.nband;
    band[i] = l;
    band[cs + i] = u[0];
    band[2 * cs + i] = u[1];
    band[3 * cs + i] = u[2];
    if (y == 0 || y == E.NY - 1) {
        const double ny = y == 0 ? -1.0 : 1.0;
        inc0[((long long)(y == 0 ? 0 : 1) * E.nz + z) * E.NX + x] = ny * u[1] - CS * l;
    }
}

// (log rho, u) of the pre-collision populations the stream gives the band
// cells inside the ring: the pull of the stored, boundary-processed ones
template <typename S>
__global__ void k_ext_band_pull(const S *__restrict__ src, Grid G, ExtGeom E, double *__restrict__ band) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)E.nband * E.nz) return;
    const int z = (int)(i / E.nband), b = (int)(i - (long long)z * E.nband);
    int x, y;
    band_cell(E, b, x, y);
    if (on_ring(E, x, y)) return;
    double d = 0.0, j[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const double g = load_g(src, G, q, x - cx(q), y - cy(q), G.wrapz(z - cz(q)));
        d += g;
        j[0] += cx(q) * g;
        j[1] += cy(q) * g;
        j[2] += cz(q) * g;
    }
    const double rho = 1.0 + d;
    const long long cs = (long long)E.nz * E.nband;
    band[i] = log(rho);
    band[cs + i] = j[0] / rho;
    band[2 * cs + i] = j[1] / rho;
    band[3 * cs + i] = j[2] / rho;
}

// one SSP-RK3 stage of the ring state (exterior.py:138-144): stage 1 from the
// band's ring values y0, stage 2 and 3 from the previous stage's values;
// stage 1 also clears the step's reconstruction moment error
__global__ void k_ext_stage(ExtGeom E, const double *__restrict__ band, const double *__restrict__ prev,
                            double *__restrict__ out, int stage, const double *__restrict__ clock,
                            const double *__restrict__ inc0, double *__restrict__ moment_error) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const double step = *clock;  // steps done before this one
    if (stage == 1 && i == 0) *moment_error = 0.0;  // the ring kernel of this step takes its maximum
    if (i >= (long long)E.nring * E.nz) return;
    const int z = (int)(i / E.nring), r = (int)(i - (long long)z * E.nring);
    int x, y;
    ring_cell(E, r, x, y);
    const RingPoint p = ring_point(E, x, y, z);
    const ExtState St{prev, band};
    double y0[4], yp[4], k[4], yn[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        y0[c] = band[((long long)c * E.nz + z) * E.nband + band_index(E, x, y)];
        yp[c] = prev ? prev[(long long)c * E.nz * E.nring + i] : y0[c];
    }
    ring_rhs(E, St, p, yp, k);
    double time = step + 1.0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        if (stage == 1)
            yn[c] = y0[c] + k[c];
        else if (stage == 2)
            yn[c] = 0.75 * y0[c] + 0.25 * (yp[c] + k[c]);
        else
            yn[c] = (y0[c] + 2 * (yp[c] + k[c])) / 3;
    }
    if (stage == 2) time = step + 0.5;
    ring_enforce(E, p, time, inc0, yn);
#pragma unroll
    for (int c = 0; c < 4; ++c) out[(long long)c * E.nz * E.nring + i] = yn[c];
}

// regularised zero-centred populations of (log rho, u) with the velocity
// gradient gv[a][b] = d u_b / d x_a (exterior.py:153-171): the product-form
// equilibrium plus the Navier-Stokes stress through the derivatives of its
// one-dimensional factors
__device__ __forceinline__ void regularized_populations(double l, const double u[3], const double gv[3][3],
                                                        double omega, double g[Q]) {
    const double rho = exp(l);
    const double div = (gv[0][0] + gv[1][1]) + gv[2][2];
    const double iso = 2.0 / 3.0 * div * (1.0 - 1.0 / omega);
    double s[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b)
            s[a][b] = (-rho / 3) * ((gv[a][b] + gv[b][a]) / omega + (a == b ? iso : 0.0));
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const double c[3] = {(double)cx(q), (double)cy(q), (double)cz(q)};
        double phi[3], first[3], second[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const double v = u[a];
            phi[a] = (2.0 / 3.0 - v * v + (1.5 * v * v - 0.5) * c[a] * c[a]) + c[a] * v / 2;
            first[a] = (-2 * v + 3 * v * c[a] * c[a]) + c[a] / 2;
            second[a] = 1.5 * c[a] * c[a] - 1;
        }
        double v = rho * (phi[0] * phi[1] * phi[2]) - weight(q);
        v += s[0][0] * second[0] * (phi[1] * phi[2]);
        v += s[1][1] * second[1] * (phi[0] * phi[2]);
        v += s[2][2] * second[2] * (phi[0] * phi[1]);
        v += s[0][1] * first[0] * first[1] * phi[2];
        v += s[0][2] * first[0] * first[2] * phi[1];
        v += s[1][2] * first[1] * first[2] * phi[0];
        g[q] = v;
    }
}

// every ring cell: rebuilt populations of the predicted state y3 with the
// gradients of the next state (ring: y3, inside: band), minus what the stream
// would have given it (pulls of src; outside the storage the freestream UBB's
// reflection, g_inv(q) - 6 (c_inv(q).U) w rho, solver.py:131 as lbmpy applies
// it in the ghost layer) summed into the exterior source (mass, momentum);
// the rebuilt state's macros go to the band for the next step, and its
// collision into dst.  moment_error receives the largest departure of the
// rebuilt set's mass and momentum from the predicted rho, rho u
// (exterior.py:168-170), as a maximum over non-negative doubles ordered by
// their bit patterns (a NaN orders above every number and is kept)
template <typename S>
__global__ void __launch_bounds__(128)
    k_ext_ring(const S *__restrict__ src, S *__restrict__ dst, Grid G, ExtGeom E, double *__restrict__ band,
               const double *__restrict__ y3, Shift27 shift, typename Store<S>::T omega_s,
               typename Store<S>::T omega_b, double omega, double *__restrict__ partials,
               double *__restrict__ moment_error) {
    using T = typename Store<S>::T;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    unsigned long long err_bits = 0ull;
    if (i < (long long)E.nring * E.nz) {
        const int z = (int)(i / E.nring), r = (int)(i - (long long)z * E.nring);
        int x, y;
        ring_cell(E, r, x, y);
        const RingPoint p = ring_point(E, x, y, z);
        const ExtState St{y3, band};
        double grad[3][4];
        ring_gradient(E, St, p, grad);
        double gv[3][3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) gv[a][b] = grad[a][1 + b];
        const long long cs = (long long)E.nz * E.nring;
        const double u[3] = {y3[cs + i], y3[2 * cs + i], y3[3 * cs + i]};
        double g[Q];
        regularized_populations(y3[i], u, gv, omega, g);
        // the streamed populations this replaces
        double here[Q], d_here = 0.0;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            here[q] = load_g(src, G, q, x, y, z);
            d_here += here[q];
        }
        const double rho_here = d_here + 1.0;
        double d = 0.0, j[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const int xs = x - cx(q), ys = y - cy(q);
            double old;
            if (xs >= 0 && xs < E.NX && ys >= 0 && ys < E.NY) {
                old = load_g(src, G, q, xs, ys, G.wrapz(z - cz(q)));
            } else {
                const int di = inv(q);
                const double term = 6.0 * (cx(di) * E.speed) * weight(di);
                old = here[di] - term * rho_here;
            }
            const double dm = g[q] - old;
            acc[0] += dm;
            acc[1] += cx(q) * dm;
            acc[2] += cy(q) * dm;
            acc[3] += cz(q) * dm;
            d += g[q];
            j[0] += cx(q) * g[q];
            j[1] += cy(q) * g[q];
            j[2] += cz(q) * g[q];
        }
        const double rho = 1.0 + d;
        {
            const double rho_p = exp(y3[i]);
            double err = fabs(rho - rho_p);
#pragma unroll
            for (int a = 0; a < 3; ++a) err = fmax(err, fabs(j[a] - rho_p * u[a]));
            if (err != err) err = __longlong_as_double(0x7ff8000000000000ll);
            err_bits = (unsigned long long)__double_as_longlong(err);
        }
        const long long bc = (long long)E.nz * E.nband, bi = (long long)z * E.nband + band_index(E, x, y);
        band[bi] = log(rho);
        band[bc + bi] = j[0] / rho;
        band[2 * bc + bi] = j[1] / rho;
        band[3 * bc + bi] = j[2] / rho;
        T t[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) t[q] = T(g[q]);
        collide_stored<S>(t, omega_s, omega_b);
        const long long cell = G.cell(x, y, z);
#pragma unroll
        for (int q = 0; q < Q; ++q) Store<S>::store(dst + q * G.qs + cell, q, t[q], shift.v[q]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long other = __shfl_down_sync(0xffffffffu, err_bits, o);
        err_bits = other > err_bits ? other : err_bits;
    }
    if ((threadIdx.x & 31) == 0 && err_bits)
        atomicMax(reinterpret_cast<unsigned long long *>(moment_error), err_bits);
    block_sum_store<4>(acc, partials);
}

// initial ring: the freestream equilibrium (solver.py:196-200)
template <typename S>
__global__ void k_ext_fill_ring(S *__restrict__ pdf, Grid G, ExtGeom E) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)E.nring * E.nz) return;
    const int z = (int)(i / E.nring), r = (int)(i - (long long)z * E.nring);
    int x, y;
    ring_cell(E, r, x, y);
    const double u[3] = {E.speed, 0.0, 0.0};
    double g[Q];
    equilibrium_g(1.0, u, g);
    for (int q = 0; q < Q; ++q) store_g(pdf, G, q, x, y, z, g[q]);
}

// collision of the stored ring populations in place (the initial state)
template <typename S>
__global__ void __launch_bounds__(128) k_ext_collide_ring(S *__restrict__ pdf, Grid G, ExtGeom E, Shift27 shift,
                                                          typename Store<S>::T omega_s, typename Store<S>::T omega_b) {
    using T = typename Store<S>::T;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)E.nring * E.nz) return;
    const int z = (int)(i / E.nring), r = (int)(i - (long long)z * E.nring);
    int x, y;
    ring_cell(E, r, x, y);
    const long long cell = G.cell(x, y, z);
    T g[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) g[q] = Store<S>::load(pdf + q * G.qs + cell, q, shift.v[q]);
    collide_stored<S>(g, omega_s, omega_b);
#pragma unroll
    for (int q = 0; q < Q; ++q) Store<S>::store(pdf + q * G.qs + cell, q, g[q], shift.v[q]);
}

// ring populations <-> (ring cell, z, 27) doubles, for checkpoints
template <typename S>
__global__ void k_ext_ring_export(const S *__restrict__ pdf, Grid G, ExtGeom E, double *__restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)E.nring * E.nz) return;
    const int z = (int)(i / E.nring), r = (int)(i - (long long)z * E.nring);
    int x, y;
    ring_cell(E, r, x, y);
    for (int q = 0; q < Q; ++q) out[i * Q + q] = load_g(pdf, G, q, x, y, z);
}
template <typename S>
__global__ void k_ext_ring_import(S *__restrict__ pdf, Grid G, ExtGeom E, const double *__restrict__ in) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)E.nring * E.nz) return;
    const int z = (int)(i / E.nring), r = (int)(i - (long long)z * E.nring);
    int x, y;
    ring_cell(E, r, x, y);
    for (int q = 0; q < Q; ++q) store_g(pdf, G, q, x, y, z, in[i * Q + q]);
}

// the validity guards also cover the ring (solver.py:289-292 reads every
// storage fluid cell): rows in k_diagnostics' layout with no density sum
template <typename S>
__global__ void __launch_bounds__(256) k_ext_ring_diagnostics(const S *__restrict__ pdf, Grid G, ExtGeom E,
                                                              double *__restrict__ partials) {
    double mx_u2 = 0.0, mx_dr = 0.0, mx_neg = -1e300, bad = 0.0;
    const long long n = (long long)E.nring * E.nz;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int z = (int)(i / E.nring), r = (int)(i - (long long)z * E.nring);
        int x, y;
        ring_cell(E, r, x, y);
        double rho, u[3];
        macro_at(pdf, G, x, y, z, rho, u);
        const double u2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
        if (!isfinite(rho) || !isfinite(u2)) {
            bad += 1.0;
            continue;
        }
        mx_u2 = fmax(mx_u2, u2);
        mx_dr = fmax(mx_dr, fabs(rho - 1.0));
        mx_neg = fmax(mx_neg, -rho);
    }
    __shared__ double red[32][4];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        mx_u2 = fmax(mx_u2, __shfl_down_sync(0xffffffffu, mx_u2, o));
        mx_dr = fmax(mx_dr, __shfl_down_sync(0xffffffffu, mx_dr, o));
        mx_neg = fmax(mx_neg, __shfl_down_sync(0xffffffffu, mx_neg, o));
        bad += __shfl_down_sync(0xffffffffu, bad, o);
    }
    if (lane == 0) {
        red[warp][0] = mx_u2;
        red[warp][1] = mx_dr;
        red[warp][2] = mx_neg;
        red[warp][3] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a[4] = {red[0][0], red[0][1], red[0][2], red[0][3]};
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            a[0] = fmax(a[0], red[w][0]);
            a[1] = fmax(a[1], red[w][1]);
            a[2] = fmax(a[2], red[w][2]);
            a[3] += red[w][3];
        }
        double *row = partials + blockIdx.x * 6;
        row[0] = a[0];
        row[1] = a[1];
        row[2] = a[2];
        row[3] = 0.0;
        row[4] = a[3];
        row[5] = 0.0;
    }
}

// the step's exterior source and wall mass, and their running sums:
// out[0..3] source (mass, momentum) of the step, out[4..7] accumulated,
// out[8] wall mass exchange of the step (sum over elements of the wall
// kernel's incoming-minus-outgoing column), out[9] accumulated; out[10] is
// the step's reconstruction moment error (k_ext_ring), out[11] the number of
// steps done (the predictor's clock)
__global__ void __launch_bounds__(REDUCE_THREADS)
    k_ext_final(const double *__restrict__ partials, long long nblocks, const double *__restrict__ walls,
                int n_elements, double *__restrict__ out) {
    double acc[4];
    reduce_rows<4>(partials, nblocks, 0u, acc);
    if (threadIdx.x == 0) {
        for (int k = 0; k < 4; ++k) {
            out[k] = acc[k];
            out[4 + k] += acc[k];
        }
        double wall = 0.0;
        for (int e = 0; e < n_elements; ++e) wall += walls[5 * e + 4];
        out[8] = wall;
        out[9] += wall;
        out[11] += 1.0;  // the step clock
    }
}

}  // namespace ak
