// ak_geometry.cuh -- solid flags, cut links and Bouzidi fractions on the GPU.
//
// These reproduce the reference's numpy geometry bit for bit
// (src/aerokinetic/geometry.py:58-85 and solver.py:93-122): every floating
// operation is issued as an individually rounded IEEE operation
// (__dadd_rn/__dsub_rn/__dmul_rn/__ddiv_rn, never contracted into an FMA) in
// the same order numpy evaluates the expression, so the flag of every column
// and the fraction of every link equal the reference's exactly.
#pragma once
#include "ak_kernels.cuh"

namespace ak {

struct Polygons {
    const double *xy;   // all vertices, (x, y) pairs
    const int *start;   // first vertex of each element
    const int *count;   // vertices of each element
    int n;
};

// even-odd crossing test, geometry.py:58-68
__device__ bool poly_contains(const double *xy, int n, double px, double py) {
    bool inside = false;
    for (int i = 0; i < n; ++i) {
        const int j = i + 1 == n ? 0 : i + 1;
        const double ax = xy[2 * i], ay = xy[2 * i + 1], bx = xy[2 * j], by = xy[2 * j + 1];
        if (by == ay) continue;
        const bool straddles = (ay > py) != (by > py);
        const double crossing =
            __dadd_rn(__ddiv_rn(__dmul_rn(__dsub_rn(bx, ax), __dsub_rn(py, ay)), __dsub_rn(by, ay)), ax);
        inside ^= straddles && (px < crossing);
    }
    return inside;
}

// cell centre of padded index X: ((X - 1) + 0.5) * dx + origin
__device__ __forceinline__ double centre(int X, double dx, double origin) {
    return __dadd_rn(__dmul_rn((double)(X - 1) + 0.5, dx), origin);
}

// flags of every padded column; later elements replace earlier ones
__global__ void k_flags(uint8_t *__restrict__ flags, int nx, int ny, Polygons P, double dx, double ox, double oy) {
    const int X = blockIdx.x * blockDim.x + threadIdx.x, Y = blockIdx.y;
    if (X >= nx + 2) return;
    const double px = centre(X, dx, ox), py = centre(Y, dx, oy);
    uint8_t f = (X == 0 || Y == 0 || X == nx + 1 || Y == ny + 1) ? FLAG_OUTER : FLAG_FLUID;
    for (int e = 0; e < P.n; ++e)
        if (poly_contains(P.xy + 2 * P.start[e], P.count[e], px, py)) f = (uint8_t)(e + 1);
    flags[(long long)Y * (nx + 2) + X] = f;
}

// link_fraction (geometry.py:70-85) and the half-way fallback
// (solver.py:113-119) for each key; status[k] = 1 when no crossing exists
__global__ void k_wall_fractions(const WallKey *__restrict__ keys, long long nkeys, Polygons P, double dx, double ox,
                                 double oy, double *__restrict__ q_out, int *__restrict__ status) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nkeys) return;
    const WallKey key = keys[k];
    const double px = centre(key.x, dx, ox), py = centre(key.y, dx, oy);
    const double offx = __dmul_rn((double)cx(key.d2), dx), offy = __dmul_rn((double)cy(key.d2), dx);
    const double *xy = P.xy + 2 * P.start[key.element];
    const int n = P.count[key.element];
    const double lo = -1e-10, hi = 1 + 1e-10;
    double q = INFINITY;
    for (int i = 0; i < n; ++i) {
        const int j = i + 1 == n ? 0 : i + 1;
        const double ax = xy[2 * i], ay = xy[2 * i + 1];
        const double ex = __dsub_rn(xy[2 * j], ax), ey = __dsub_rn(xy[2 * j + 1], ay);
        const double den = __dsub_rn(__dmul_rn(offx, ey), __dmul_rn(offy, ex));
        if (!(fabs(den) > 1e-14)) continue;
        const double rx = __dsub_rn(ax, px), ry = __dsub_rn(ay, py);
        const double t = __ddiv_rn(__dsub_rn(__dmul_rn(rx, ey), __dmul_rn(ry, ex)), den);
        const double v = __ddiv_rn(__dsub_rn(__dmul_rn(rx, offy), __dmul_rn(ry, offx)), den);
        if (t >= lo && t <= hi && v >= lo && v <= hi) q = fmin(q, t);
    }
    if (!isfinite(q)) {
        status[k] = 1;
        q_out[k] = 0.0;
        return;
    }
    q = fmin(fmax(q, 1e-10), 1.0);
    const double qx = __dsub_rn(px, offx), qy = __dsub_rn(py, offy);
    bool blocked = false;
    for (int e = 0; e < P.n; ++e) blocked |= poly_contains(P.xy + 2 * P.start[e], P.count[e], qx, qy);
    if (q < 0.5 && blocked) q = -1.0;
    q_out[k] = q;
    status[k] = 0;
}

}  // namespace ak
