// ak_kernels.cuh -- sm_103a kernels of the uniform engine.
//
// HBM layout of one case (all device-resident for the life of the case):
//   populations  two copies (A/B), structure of arrays pdf[q][z][y][x]; x and
//                y carry one ghost layer (x, y in 0..n+1), z is periodic and
//                wraps in the index arithmetic; rows are padded to a multiple
//                of 32 elements.  Storage double, float or half.
//   flags        one byte per padded (x, y) column: 0 fluid, k+1 wall element
//                k, 255 outer ghost.  The geometry is extruded, so a column
//                flag covers the whole span and stays in L2.
//   wall keys    compacted (x, y, planar direction, element) + Bouzidi q;
//                one key stands for nz * 3 links (all z and all c_z).
//   outer links  (x, y, z, d, boundary object) of the links into the ghost
//                ring, with the per-link state of the legacy outflow or the
//                characteristic farfield.
//
// One step (the reference's solver.py:256-261) is, on the case's stream:
//   outer boundary kernels -> wall kernel (Bouzidi into solid cells, loads)
//   -> stream_collide (pull from A, collide, write B) -> swap A/B.
#pragma once
#include <type_traits>

#include "ak_lattice.cuh"

namespace ak {

constexpr uint8_t FLAG_FLUID = 0;
constexpr uint8_t FLAG_OUTER = 255;
constexpr double CS = 0.57735026918962576451;
constexpr double ONE_MINUS_CS = 0.42264973081037423549;

struct Grid {
    int nx, ny, nz;   // interior
    int nxp, nyp;     // padded columns
    int sx;           // row pitch (elements)
    long long plane;  // nyp * sx
    long long qs;     // nz * plane, stride between populations
    const float *shift;  // FP16 storage: zero-centred freestream equilibrium per direction (device)
    __host__ __device__ long long cell(int x, int y, int z) const { return (long long)z * plane + (long long)y * sx + x; }
    __device__ int wrapz(int z) const { return z < 0 ? z + nz : (z >= nz ? z - nz : z); }
};

#ifdef AK_CHECKED
// Debug builds check every population index against the padded lattice and
// record the first offending access (kernel tag, q, x, y, z) instead of
// performing it.
__device__ unsigned long long ak_debug_word;
__device__ __forceinline__ bool ak_in_range(const Grid &G, int q, int x, int y, int z, int tag) {
    if (q >= 0 && q < Q && x >= 0 && x < G.nxp && y >= 0 && y < G.nyp && z >= 0 && z < G.nz) return true;
    const unsigned long long code = 1ULL << 63 | (unsigned long long)(tag & 0xff) << 48 |
                                    (unsigned long long)(q & 0xff) << 40 | (unsigned long long)(x & 0xfff) << 28 |
                                    (unsigned long long)(y & 0xfff) << 16 | (unsigned long long)(z & 0xffff);
    atomicCAS(&ak_debug_word, 0ULL, code);
    return false;
}
#define AK_CHECK(G, q, x, y, z, tag) ak_in_range(G, q, x, y, z, tag)
#else
#define AK_CHECK(G, q, x, y, z, tag) true
#endif

// Kernels of the two-level step's chains may be launched with programmatic
// stream serialization (launch_chained on the host): such a launch can be
// scheduled while its predecessor on the stream drains, and waits here,
// before it touches memory, until that predecessor has completed and its
// writes are visible.  Launched the ordinary way, the wait returns at once.
__device__ __forceinline__ void chain_wait() {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
    asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
}

template <typename S>
__device__ __forceinline__ double load_g(const S *pdf, const Grid &G, int q, int x, int y, int z) {
    if (!AK_CHECK(G, q, x, y, z, 1)) return 0.0;
    return (double)Store<S>::load(pdf + q * G.qs + G.cell(x, y, z), q, G.shift[q]);
}
template <typename S>
__device__ __forceinline__ void store_g(S *pdf, const Grid &G, int q, int x, int y, int z, double v) {
    if (!AK_CHECK(G, q, x, y, z, 2)) return;
    Store<S>::store(pdf + q * G.qs + G.cell(x, y, z), q, (typename Store<S>::T)v, G.shift[q]);
}

// ------------------------------------------------------------ bulk step
// shift of direction q: by value in the single-case kernel (constant bank),
// from the case's device table in the batched one
__device__ __forceinline__ float shift_at(const Shift27 &s, int q) { return s.v[q]; }
__device__ __forceinline__ float shift_at(const float *s, int q) { return __ldg(s + q); }

// Validity and conservation statistics of a set of cells, in this order
// (the layout the two-level budget reduces): max |u|^2, max |rho - 1|,
// sum drho, sum j (3), cells, non-finite cells.
constexpr int CELL_STATS = 8;

// The budget's sums on the integer pipe.  A value v becomes the integer
// round(v 2^FIX_BITS) (magnitude rounded half up, then the sign): integer
// sums are exact, so a row's sum does not depend on the order of its cells,
// and the FP64-bound passes spend no FP64 instruction on them (GB300 issues
// an FP64 instruction per warp at 1/64 of the FP32 rate).  A value that is
// not finite, or whose magnitude reaches 2^MAX_EXP, is refused.
constexpr int FIX_BITS = 50;
constexpr double FIX_UNIT = 1.0 / 1125899906842624.0;  // 2^-FIX_BITS
// |result| < 2^(FIX_BITS + MAX_EXP)
template <int MAX_EXP>
__device__ __forceinline__ bool fixed_of(double v, long long &out) {
    const long long b = __double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e == 0x7ff || e > 1022 + MAX_EXP) return false;
    long long r = 0;
    if (e != 0) {
        const long long m = (b & 0x000fffffffffffffLL) | 0x0010000000000000LL;  // v = m 2^(e - 1075)
        const int sh = e - 1075 + FIX_BITS;
        if (sh >= 0)
            r = m << sh;
        else if (sh > -55)
            r = (m + (1LL << (-sh - 1))) >> -sh;
    }
    out = b < 0 ? -r : r;
    return true;
}
template <int MAX_EXP>
__device__ __forceinline__ bool fixed_of(float v, long long &out) {
    const int b = __float_as_int(v);
    const int e = (b >> 23) & 0xff;
    if (e == 0xff || e > 126 + MAX_EXP) return false;
    long long r = 0;
    if (e != 0) {
        const long long m = (b & 0x7fffff) | 0x800000;  // v = m 2^(e - 150)
        const int sh = e - 150 + FIX_BITS;
        if (sh >= 0)
            r = m << sh;
        else if (sh > -26)
            r = (m + (1LL << (-sh - 1))) >> -sh;
    }
    out = b < 0 ? -r : r;
    return true;
}
template <int MAX_EXP>
__device__ __forceinline__ bool fixed_of(df64 v, long long &out) {
    long long hi, lo;
    if (!fixed_of<MAX_EXP>(v.hi, hi) || !fixed_of<MAX_EXP>(v.lo, lo)) return false;
    out = hi + lo;
    return true;
}

// The budget's row of a set of cells, in the CELL_STATS layout (the maxima,
// which only the diagnostics use, are left 0): drho and j summed as fixed
// point (each value below 256 in magnitude, so that 32 cells' sums stay
// inside 64 bits), fluid cells and invalid cells counted.
struct BudgetSums {
    long long drho = 0, jx = 0, jy = 0, jz = 0;
    int cells = 0, bad = 0;
    template <typename T>
    __device__ __forceinline__ void add_cell(T drho_, T jx_, T jy_, T jz_) {
        long long a, b, c, d;
        if (fixed_of<8>(drho_, a) && fixed_of<8>(jx_, b) && fixed_of<8>(jy_, c) && fixed_of<8>(jz_, d)) {
            drho += a;
            jx += b;
            jy += c;
            jz += d;
            ++cells;
        } else {
            ++bad;
        }
    }
};
// the warp's sum of a 64-bit value whose 32-lane sum fits in 64 bits, by
// three warp-reduce instructions: v = p2 2^54 + p1 2^27 + p0 with p0, p1 in
// [0, 2^27) (32 of them sum below 2^32) and p2 = v >> 54; the parts' sums
// are recombined modulo 2^64, which is exact when the sum fits
__device__ __forceinline__ long long warp_sum_fixed(long long v) {
    const unsigned long long u = (unsigned long long)v;
    const unsigned s0 = __reduce_add_sync(0xffffffffu, (unsigned)(u & 0x7ffffffULL));
    const unsigned s1 = __reduce_add_sync(0xffffffffu, (unsigned)((u >> 27) & 0x7ffffffULL));
    const int s2 = __reduce_add_sync(0xffffffffu, (int)(v >> 54));
    return (long long)(((unsigned long long)(long long)s2 << 54) + ((unsigned long long)s1 << 27) + s0);
}
// the warp's row (every lane calls it; no block-wide barrier): integer warp
// sums, written as integers (drho, jx, jy, jz, fluid cells, invalid cells in
// the first six of the row's CELL_STATS slots).  A conversion to double here
// puts FP64 instructions at the end of every warp of an FP64-bound pass,
// where they queue behind the collisions and hold the block: converting in
// the warp made the two-level budget step 1.178 ms, converting in the
// reduction 1.145 ms (bare step 1.113 ms); the reduction converts them
__device__ __forceinline__ void warp_budget_row(BudgetSums s, long long *out, long long row) {
    s.drho = warp_sum_fixed(s.drho);
    s.jx = warp_sum_fixed(s.jx);
    s.jy = warp_sum_fixed(s.jy);
    s.jz = warp_sum_fixed(s.jz);
    s.cells = __reduce_add_sync(0xffffffffu, s.cells);
    s.bad = __reduce_add_sync(0xffffffffu, s.bad);
    if ((threadIdx.x & 31) == 0) {
        long long *r = out + row * CELL_STATS;
        r[0] = s.drho;
        r[1] = s.jx;
        r[2] = s.jy;
        r[3] = s.jz;
        r[4] = s.cells;
        r[5] = s.bad;
    }
}
// a budget row as the CELL_STATS doubles (maxima 0)
__device__ __forceinline__ void budget_row_values(const long long *__restrict__ r, double (&v)[CELL_STATS]) {
    v[0] = 0.0;
    v[1] = 0.0;
#pragma unroll
    for (int k = 0; k < 4; ++k) v[2 + k] = (double)r[k] * FIX_UNIT;
    v[6] = (double)r[4];
    v[7] = (double)r[5];
}

// pull the 27 populations of interior cell (x, y, z) (padded x, y), collide,
// store into dst if the column is fluid; stream_only: store the pulled values
// as they are (bit copies, no collision); mac (optional): where the
// collision writes the cell's drho and j.  Returns true for a collided fluid
// cell.
template <typename S, typename Shift>
__device__ __forceinline__ bool stream_collide_cell(const S *__restrict__ src, S *__restrict__ dst,
                                                    const uint8_t *__restrict__ flags, const Grid &G,
                                                    const Shift &shift, typename Store<S>::T omega_s,
                                                    typename Store<S>::T omega_b, int x, int y, int z,
                                                    const Sgs<typename Store<S>::T> &sgs,
                                                    bool stream_only = false, typename Store<S>::T *mac = nullptr) {
    using T = typename Store<S>::T;
    // the column flag only gates the stores, so the 27 loads issue at once
    const bool fluid = __ldg(flags + y * G.nxp + x) == FLAG_FLUID;
    // the cell's column in the three z planes it pulls from; a direction adds
    // q * qs - cy * sx - cx, so each load costs one address add
    const S *row[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) row[c] = src + (long long)G.wrapz(z - (c - 1)) * G.plane + (long long)y * G.sx + x;
    if (stream_only) {
        if (!fluid) return false;
        const long long c = G.cell(x, y, z);
#pragma unroll
        for (int q = 0; q < Q; ++q)
            dst[q * G.qs + c] = row[cz(q) + 1][(long long)q * G.qs - (long long)cy(q) * G.sx - cx(q)];
        return false;
    }
    T g[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const long long off = (long long)q * G.qs - (long long)cy(q) * G.sx - cx(q);
        g[q] = AK_CHECK(G, q, x - cx(q), y - cy(q), G.wrapz(z - cz(q)), 3)
                   ? Store<S>::load(row[cz(q) + 1] + off, q, shift_at(shift, q))
                   : T(0);
    }
    collide_stored<S>(g, omega_s, omega_b, sgs, mac);
    if (!fluid) return false;
    const long long c = G.cell(x, y, z);
#pragma unroll
    for (int q = 0; q < Q; ++q) Store<S>::store(dst + q * G.qs + c, q, g[q], shift_at(shift, q));
    return true;
}

// ------------------------------------------------------------ cell pairs
// The FP32-compute storage forms advance two x-adjacent cells (xe, xe + 1),
// xe even in padded coordinates, per thread: the collision of both runs as
// one stream of packed FP32x2 instructions (ak_f32x2.cuh), the populations
// that stay in their column (c_x = 0) are read as one aligned 4- or 8-byte
// pair, and both cells' stores go out as pairs.  Rows, planes and the
// population stride are even, so xe even keeps every pair aligned.
template <typename S>
__host__ __device__ constexpr bool pair_form() {
    return std::is_same_v<S, float> || std::is_same_v<S, __half>;
}
// the pair of values at p, p + 1 as FP32 (p at an even element)
__device__ __forceinline__ float2 load_pair(const float *p) { return __ldg(reinterpret_cast<const float2 *>(p)); }
__device__ __forceinline__ float2 load_pair(const __half *p) {
    return __half22float2(__ldg(reinterpret_cast<const __half2 *>(p)));
}
__device__ __forceinline__ float load_one(const float *p) { return __ldg(p); }
__device__ __forceinline__ float load_one(const __half *p) { return __half2float(__ldg(p)); }
__device__ __forceinline__ void store_pair(float *p, float2 v) { *reinterpret_cast<float2 *>(p) = v; }
__device__ __forceinline__ void store_pair(__half *p, float2 v) {
    *reinterpret_cast<__half2 *>(p) = __float22half2_rn(v);
}
__device__ __forceinline__ void store_one(float *p, float v) { *p = v; }
__device__ __forceinline__ void store_one(__half *p, float v) { *p = __float2half_rn(v); }

// items of one stream-collide launch over the padded columns rect (rect.y ==
// 0: the interior): cells, or cell pairs (xe even) for the pair forms
template <typename S>
__host__ __device__ __forceinline__ long long stream_collide_items(int4 rect, int nx, int ny, int nz) {
    if (rect.y == 0) rect = make_int4(1, nx + 1, 1, ny + 1);
    const long long h = rect.w - rect.z;
    if constexpr (pair_form<S>()) return (long long)((((rect.y + 1) & ~1) - (rect.x & ~1)) / 2) * h * nz;
    return (long long)(rect.y - rect.x) * h * nz;
}

// The 27 pulled populations of a cell pair as loaded: FP16 pairs packed in
// one 32-bit word each, FP32 pairs as float2.
template <typename S> struct PairRaw;
template <> struct PairRaw<__half> { unsigned v[Q]; };
template <> struct PairRaw<float> { float2 v[Q]; };

// Cells xe + k of row (y, z), k = 0, 1, with live[k] set when the cell
// belongs to the launch (only a live cell's pulls are read): the pulls of
// both, the c_x = 0 ones as one aligned pair
template <typename S>
__device__ __forceinline__ void pair_load(const S *__restrict__ src, const Grid &G, int xe, int y, int z, bool live0,
                                          bool live1, PairRaw<S> &raw) {
    const S *row[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) row[c] = src + (long long)G.wrapz(z - (c - 1)) * G.plane + (long long)y * G.sx + xe;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const S *p = row[cz(q) + 1] + ((long long)q * G.qs - (long long)cy(q) * G.sx);
        if constexpr (std::is_same_v<S, __half>) {
            // p is at xe: every load is an aligned 32-bit word; a shifted
            // pair (xe - cx, xe + 1 - cx) is the upper half of one word and
            // the lower half of the next, put together by one byte permute
            const unsigned *w = reinterpret_cast<const unsigned *>(p);
            if (cx(q) == 0) {
                raw.v[q] = __ldg(w);
            } else if (cx(q) > 0) {
                const unsigned left = live0 ? __ldg(w - 1) : 0u, own = live1 ? __ldg(w) : 0u;
                raw.v[q] = __byte_perm(left, own, 0x5432);
            } else {
                const unsigned own = live0 ? __ldg(w) : 0u, right = live1 ? __ldg(w + 1) : 0u;
                raw.v[q] = __byte_perm(own, right, 0x5432);
            }
        } else {
            if (cx(q) == 0) {
                raw.v[q] = __ldg(reinterpret_cast<const float2 *>(p));
            } else {
                raw.v[q].x = live0 ? __ldg(p - cx(q)) : 0.0f;
                raw.v[q].y = live1 ? __ldg(p + 1 - cx(q)) : 0.0f;
            }
        }
    }
}

// population q of both cells as stored: FP16 storage holds (f - w - shift) / w
template <typename S, typename Shift>
__device__ __forceinline__ float2 stored_pair(F2 g, const Shift &shift, int q) {
    if constexpr (std::is_same_v<S, __half>) {
        const float a = shift_at(shift, q), inv = (float)(1.0 / weight(q)), b = -a * inv;
        return f2_fma(g.v, make_float2(inv, inv), make_float2(b, b));
    } else {
        return g.v;
    }
}

// The collision of both cells in packed FP32x2 and their stores (fluid
// cells only; a pair of stores where both are).  Each lane rounds as the
// one-cell path's FP32 operations do, except that the collision's
// multiply-add contractions are this code's own.
template <typename S, typename Shift>
__device__ __forceinline__ void pair_collide_store(const PairRaw<S> &raw, S *__restrict__ dst,
                                                   const uint8_t *__restrict__ flags, const Grid &G,
                                                   const Shift &shift, float omega_s, float omega_b, int xe, int y,
                                                   int z, bool live0, bool live1, const Sgs<F2> &sgs) {
    const bool store0 = live0 && __ldg(flags + y * G.nxp + xe) == FLAG_FLUID;
    const bool store1 = live1 && __ldg(flags + y * G.nxp + xe + 1) == FLAG_FLUID;
    // the store address and stride formed before the collision: two values
    // held across it instead of the lattice geometry (the batch kernel reads
    // that from its case descriptor, not from launch parameters)
    S *const p = dst + G.cell(xe, y, z);
    const long long qs = G.qs;
    F2 g[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        if constexpr (std::is_same_v<S, __half>) {
            __half2 h;
            memcpy(&h, &raw.v[q], sizeof h);
            const float w = (float)weight(q), a = shift_at(shift, q);
            g[q] = F2(f2_fma(__half22float2(h), make_float2(w, w), make_float2(a, a)));
        } else {
            g[q] = F2(raw.v[q]);
        }
    }
    if constexpr (sizeof(S) == sizeof(float))
        collide<F2>(g, F2(omega_s), F2(omega_b), sgs);
    else
        collide_full<F2>(g, F2(1.0f - omega_s), F2(omega_b), sgs);
    if (!store0 && !store1) return;
    // one branch for the pair: both cells stored (all but boundary pairs),
    // or each on its own
    if (store0 && store1) {
#pragma unroll
        for (int q = 0; q < Q; ++q) store_pair(p + q * qs, stored_pair<S>(g[q], shift, q));
    } else {
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const float2 v = stored_pair<S>(g[q], shift, q);
            if (store0) store_one(p + q * qs, v.x);
            if (store1) store_one(p + q * qs + 1, v.y);
        }
    }
}

// item i of a pair-form launch over the padded columns rect (rect.y != 0):
// pairs (xe, xe + 1), xe even, covering the columns [rect.x, rect.y) of each
// row, x fastest, then y, then z.  False when i lies beyond the launch or
// neither cell belongs to it.
struct PairItem {
    int xe, y, z;
    bool live0, live1, only;  // only: a cell is streamed without collision
};
__device__ __forceinline__ bool pair_item(const Grid &G, int4 raw, int4 rect, int4 skip, long long i, PairItem &it) {
    const int xa = rect.x & ~1;
    // a row holds at most 16384 pairs and a plane at most 2^30 (the case
    // limits), so 32-bit divisions serve every index below 2^32
    const unsigned wp = (unsigned)((((rect.y + 1) & ~1) - xa) / 2), nxy = wp * (unsigned)(rect.w - rect.z);
    if (i >= (long long)nxy * G.nz) return false;
    unsigned z, r;
    if (i < (1LL << 32)) {
        z = (unsigned)i / nxy;
        r = (unsigned)i - z * nxy;
    } else {
        z = (unsigned)(i / nxy);
        r = (unsigned)(i - (long long)z * nxy);
    }
    const unsigned yr = r / wp;
    it.z = (int)z;
    it.xe = xa + 2 * (int)(r - yr * wp);
    it.y = rect.z + (int)yr;
    bool live[2], only = false;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const int x = it.xe + k;
        live[k] = x >= rect.x && x < rect.y && !(x >= skip.x && x < skip.y && it.y >= skip.z && it.y < skip.w);
        only |= live[k] && x >= raw.x && x < raw.y && it.y >= raw.z && it.y < raw.w;
    }
    it.live0 = live[0];
    it.live1 = live[1];
    it.only = only;
    return live[0] || live[1];
}

// one pair without prefetch; a pair with a streamed-only cell takes the
// one-cell path for both cells
template <typename S, typename Shift>
__device__ __forceinline__ void stream_collide_pair(const S *__restrict__ src, S *__restrict__ dst,
                                                    const uint8_t *__restrict__ flags, const Grid &G,
                                                    const Shift &shift, float omega_s, float omega_b,
                                                    const Sgs<float> &sgs, int4 raw, const PairItem &it) {
    if (it.only) {
        for (int k = 0; k < 2; ++k) {
            const int x = it.xe + k;
            if (!(k ? it.live1 : it.live0)) continue;
            const bool only = x >= raw.x && x < raw.y && it.y >= raw.z && it.y < raw.w;
            stream_collide_cell(src, dst, flags, G, shift, omega_s, omega_b, x, it.y, it.z, sgs, only);
        }
        return;
    }
    Sgs<F2> s2;
    s2.tau0 = sgs.tau0;
    s2.c18 = sgs.c18;
    PairRaw<S> r;
    pair_load(src, G, it.xe, it.y, it.z, it.live0, it.live1, r);
    pair_collide_store(r, dst, flags, G, shift, omega_s, omega_b, it.xe, it.y, it.z, it.live0, it.live1, s2);
}

// item i of a pair-form launch (one pair, no prefetch): the batch's body
template <typename S, typename Shift>
__device__ __forceinline__ void stream_collide_pair_item(const S *__restrict__ src, S *__restrict__ dst,
                                                         const uint8_t *__restrict__ flags, const Grid &G,
                                                         const Shift &shift, float omega_s, float omega_b,
                                                         const Sgs<float> &sgs, int4 raw, int4 rect, int4 skip,
                                                         long long i) {
    PairItem it;
    if (!pair_item(G, raw, rect, skip, i, it)) return;
    stream_collide_pair(src, dst, flags, G, shift, omega_s, omega_b, sgs, raw, it);
}

// resident 128-thread blocks per SM the stream-collide is compiled for: the
// pair forms hold two cells' populations per thread.  Measured on the
// uniform 768 x 512 x 8 case (CUDA events, L2 flushed): the FP16 pairs reach
// 0.54 / 0.58 / 0.60 / 0.51 of the HBM copy peak at 4 / 5 / 6 / 8 blocks
// (96 / 95 / 80 / 64 registers), the FP32 pairs 0.87 / 0.81 / 0.63 at 4 / 5 / 6.
template <typename S>
__host__ __device__ constexpr int stream_collide_min_blocks() {
    return pair_form<S>() ? (std::is_same_v<S, __half> ? 6 : 4) : Store<S>::MIN_BLOCKS;
}

// STATS: every warp also writes the budget row (warp_budget_row) of the
// cells it collided (not the streamed-only ones) to row blockIdx.x * 4 + warp
// of stats
template <typename S, bool STATS = false>
__global__ void __launch_bounds__(128, stream_collide_min_blocks<S>())
    k_stream_collide(const S *__restrict__ src, S *__restrict__ dst, const uint8_t *__restrict__ flags, Grid G,
                     Shift27 shift, typename Store<S>::T omega_s, typename Store<S>::T omega_b,
                     Sgs<typename Store<S>::T> sgs, int4 raw = make_int4(0, 0, 0, 0),
                     int4 rect = make_int4(0, 0, 0, 0), int4 skip = make_int4(0, 0, 0, 0),
                     long long *__restrict__ stats = nullptr) {
    chain_wait();
    // one thread per cell of the padded columns x [rect.x, rect.y) by y
    // [rect.z, rect.w) (rect.y == 0: the whole interior), every z, x fastest,
    // numbered across rows: warps stay full whatever the width (the plain
    // form is bound by the FP64 pipe, where a warp with a few live lanes
    // costs as much as a full one); columns inside skip are left to another
    // launch
    if (rect.y == 0) rect = make_int4(1, G.nx + 1, 1, G.ny + 1);
    if constexpr (pair_form<S>()) {
        stream_collide_pair_item(src, dst, flags, G, shift, omega_s, omega_b, sgs, raw, rect, skip,
                                 (long long)blockIdx.x * blockDim.x + threadIdx.x);
        return;
    }
    const unsigned w = (unsigned)(rect.y - rect.x), h = (unsigned)(rect.w - rect.z);
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned nxy = w * h;
    using T = typename Store<S>::T;
    T mac[4];
    bool active = i < nxy * (unsigned)G.nz, counted = false;
    int x = 0, y = 0, z = 0;
    if (active) {
        z = (int)(i / nxy);
        const unsigned r = i - (unsigned)z * nxy;
        const unsigned yr = r / w;
        x = rect.x + (int)(r - yr * w);
        y = rect.z + (int)yr;
        active = !(x >= skip.x && x < skip.y && y >= skip.z && y < skip.w);
    }
    if constexpr (!STATS) {
        if (!active) return;
    }
    if (active) {
        // raw: the padded x [raw.x, raw.y) by y [raw.z, raw.w) columns are
        // only streamed (they keep pre-collision populations)
        const bool stream_only = x >= raw.x && x < raw.y && y >= raw.z && y < raw.w;
        counted = stream_collide_cell(src, dst, flags, G, shift, omega_s, omega_b, x, y, z, sgs, stream_only,
                                      STATS ? mac : nullptr);
    }
    if constexpr (STATS) {
        BudgetSums acc;
        if (counted) acc.add_cell(mac[0], mac[1], mac[2], mac[3]);
        warp_budget_row(acc, stats, (long long)blockIdx.x * 4 + (threadIdx.x >> 5));
    }
}

// ------------------------------------------------------------ walls
struct WallKey {
    int x, y;      // padded coordinates of the fluid column
    int d2;        // direction index of (cx, cy, 0)
    int element;
};

// Block reduction of nv doubles per thread into shared partials; thread 0 of
// the block writes them to out[blockIdx.x * nv ...] in a fixed order.
template <int NV>
__device__ void block_sum_store_at(double (&v)[NV], double *out, long long block);
template <int NV>
__device__ void block_sum_store(double (&v)[NV], double *out) {
    block_sum_store_at<NV>(v, out, blockIdx.x);
}
template <int NV>
__device__ void block_sum_store_at(double (&v)[NV], double *out, long long block) {
    __shared__ double red[32][NV];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k)
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) red[warp][k] = v[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        for (int k = 0; k < NV; ++k) {
            double s = 0.0;
            for (int w = 0; w < nw; ++w) s += red[w][k];
            out[block * NV + k] = s;
        }
    }
}

// link tid of the compacted keys (nz * 3 links per key): the Bouzidi value
// stored into the solid cell, and with sample the link's load contribution
template <typename S>
__device__ __forceinline__ void wall_link(S *__restrict__ pdf, const Grid &G, const WallKey *__restrict__ keys,
                                          const double *__restrict__ qs, long long tid, int sample, double ox,
                                          double oy, double acc[5], int &element) {
    const long long k = tid / (3LL * G.nz);
    const int rem = (int)(tid - k * 3LL * G.nz);
    const int z = rem / 3, icz = rem - 3 * (rem / 3);
    const WallKey key = keys[k];
    const int ex = cx(key.d2), ey = cy(key.d2), ez = icz - 1;
    const int d = qof(ex + 1, ey + 1, icz), di = inv(d);
    const double q = qs[k];
    const double f_xf = load_g(pdf, G, d, key.x, key.y, z);
    const double f_xf_inv = load_g(pdf, G, di, key.x, key.y, z);
    double v;
    if (q >= 0.5) {
        v = (0.5 * (f_xf + f_xf_inv * (2.0 * q - 1.0))) / q;
    } else if (q > 0.0) {
        const double d_x2f = load_g(pdf, G, d, key.x - ex, key.y - ey, G.wrapz(z - ez));
        v = 2.0 * q * f_xf + (1.0 - 2.0 * q) * d_x2f;
    } else {
        v = f_xf;
    }
    store_g(pdf, G, di, key.x + ex, key.y + ey, G.wrapz(z + ez), v);
    if (sample) {
        // the stored value is what the fluid will pull; use it as g_in
        const double gin = load_g(pdf, G, di, key.x + ex, key.y + ey, G.wrapz(z + ez));
        const double s = f_xf + gin;
        const double fx = ex * s, fy = ey * s, fz = ez * s;
        const double rx = (double)(key.x - 1) + 0.5 + ox, ry = (double)(key.y - 1) + 0.5 + oy;
        acc[0] = fx;
        acc[1] = fy;
        acc[2] = fz;
        acc[3] = rx * fy - ry * fx;
        acc[4] = gin - f_xf;
        element = key.element;
    }
}

// per-element block sums of the links' load contributions:
// partials[element][block][5], nblocks blocks per element
__device__ __forceinline__ void wall_block_sums(const double acc[5], int element, int n_elements, double *partials,
                                                long long block, long long nblocks) {
    for (int e = 0; e < n_elements; ++e) {
        double v[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) v[k] = element == e ? acc[k] : 0.0;
        block_sum_store_at<5>(v, partials + (long long)e * 5 * nblocks, block);
        __syncthreads();
    }
}

// NoSlipLinearBouzidi (solver.py:139-143) over all links of the compacted keys,
// written into the solid cells of pdf; optionally the per-element loads of
// solver.py:217-243: F = sum c_d (g_out + g_in), Mz = sum rx Fy - ry Fx,
// mass = sum g_in - g_out.  Partials: [element][block][5].
constexpr int MAX_ELEMENTS = 8;

// The last block of a sampled k_walls launch to finish sums the partials as
// k_sum_partials does (the same order, so the same result) into
// out[5 n_elements]; with cum it also adds first[t] + out[t] to cum[t] (the
// running loads of a two-level step, first holding its first fine step's
// loads), in the order of a two-level step's loads.  done counts the blocks that have
// finished; the last one leaves it 0 for the next launch.
__device__ void finish_wall_sums(const double *partials, int n_elements, unsigned *done, double *out, double *cum,
                                 const double *first) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(done, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nv = 5 * n_elements, nb = gridDim.x;
    for (int t = warp; t < nv; t += blockDim.x >> 5) {
        const int e = t / 5, k = t - 5 * e;
        double v = 0.0;
        for (int b = lane; b < nb; b += 32) v += __ldcg(partials + ((long long)e * nb + b) * 5 + k);
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) {
            out[t] = v;
            if (cum) cum[t] += first[t] + v;
        }
    }
    if (threadIdx.x == 0) *done = 0;
}

// done == nullptr: the partials are left for k_sum_partials
template <typename S>
__global__ void __launch_bounds__(256, 2) k_walls(S *__restrict__ pdf, Grid G, const WallKey *__restrict__ keys,
                                               const double *__restrict__ qs, long long nkeys, int sample,
                                               int n_elements, double ox, double oy,
                                               double *__restrict__ partials, unsigned *done = nullptr,
                                               double *out = nullptr, double *cum = nullptr,
                                               const double *first = nullptr) {
    chain_wait();
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double acc[5] = {0, 0, 0, 0, 0};
    int element = -1;
    if (tid < nkeys * G.nz * 3) wall_link(pdf, G, keys, qs, tid, sample, ox, oy, acc, element);
    if (!sample) return;
    wall_block_sums(acc, element, n_elements, partials, blockIdx.x, gridDim.x);
    if (done) finish_wall_sums(partials, n_elements, done, out, cum, first);
}

// partials laid out [element][block][5]; one warp per (element, component):
// lane-strided sums combined by a fixed butterfly, so the result does not
// depend on scheduling
__global__ void k_sum_partials(const double *__restrict__ partials, int nblocks, int nvalues,
                               double *__restrict__ out) {
    const int t = blockIdx.x, lane = threadIdx.x;
    if (t >= nvalues) return;
    const int e = t / 5, k = t - 5 * (t / 5);
    double s = 0.0;
    for (int b = lane; b < nblocks; b += 32) s += partials[((long long)e * nblocks + b) * 5 + k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) out[t] = s;
}

// ------------------------------------------------------------ outer ring
struct OuterLinks {
    const int *x, *y, *z;     // padded x, y; interior z
    const signed char *d;     // direction from the fluid cell into the ghost ring
    const signed char *obj;   // boundary object (farfield: normal index)
    const signed char *edge;  // farfield: edge flag of the foot in x and y (2 per link)
    long long n;
};

// compressible UBB (solver.py:131): g_inv(x+c) = g_d(x) - 6 (c.U) w_d rho(x).
// One thread per boundary cell and z: cells[3 i] = padded x, cells[3 i + 1] =
// padded y, cells[3 i + 2] = bit mask of the cell's UBB directions; the
// density is summed once per cell, in direction order.
template <typename S>
__device__ __forceinline__ void ubb_item(S *__restrict__ pdf, const Grid &G, const int *__restrict__ cells,
                                         long long ncells, double ux, double uy, double uz, long long i) {
    const int z = (int)(i / ncells);
    const long long c = i - (long long)z * ncells;
    const int x = cells[3 * c], y = cells[3 * c + 1], mask = cells[3 * c + 2];
    double g[Q], drho = 0.0;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        g[q] = load_g(pdf, G, q, x, y, z);
        drho += g[q];
    }
    const double rho = drho + 1.0;
#pragma unroll
    for (int d = 1; d < Q; ++d) {
        if (!((mask >> d) & 1)) continue;
        const double term = 6.0 * (cx(d) * ux + cy(d) * uy + cz(d) * uz) * weight(d);
        store_g(pdf, G, inv(d), x + cx(d), y + cy(d), G.wrapz(z + cz(d)), g[d] - term * rho);
    }
}
template <typename S>
__global__ void k_ubb(S *__restrict__ pdf, Grid G, const int *__restrict__ cells, long long ncells, double ux,
                      double uy, double uz) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ncells * G.nz) return;
    ubb_item(pdf, G, cells, ncells, ux, uy, uz, i);
}

// ExtrapolationOutflow (Geier et al. 2015 eq. F.1, normal +x): first-order
// upwind advection at c_s of the incoming population on the boundary cell.
// state[2i] = neighbour value of the previous step, state[2i+1] = boundary
// value of the previous step.
template <typename S>
__device__ __forceinline__ void outflow_item(S *__restrict__ pdf, const Grid &G, const OuterLinks &L,
                                             const int *__restrict__ selected, double *__restrict__ state, int nx_,
                                             int ny_, int nz_, long long i) {
    const int li = selected[i];
    const int x = L.x[li], y = L.y[li], z = L.z[li], d = L.d[li], di = inv(d);
    const double nb = load_g(pdf, G, di, x + cx(d) - nx_, y + cy(d) - ny_, G.wrapz(z + cz(d) - nz_));
    const double v = CS * state[2 * i] + ONE_MINUS_CS * state[2 * i + 1];
    state[2 * i] = nb;
    state[2 * i + 1] = v;
    store_g(pdf, G, di, x + cx(d), y + cy(d), G.wrapz(z + cz(d)), v);
}
template <typename S>
__global__ void k_outflow(S *__restrict__ pdf, Grid G, OuterLinks L, const int *__restrict__ selected, long long n,
                          double *__restrict__ state, int nx_, int ny_, int nz_) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    outflow_item(pdf, G, L, selected, state, nx_, ny_, nz_, i);
}

// first application: neighbour value from the initial populations, boundary
// value from the zero-centred equilibrium of the initial freestream
template <typename S>
__global__ void k_outflow_prepare(const S *__restrict__ pdf, Grid G, OuterLinks L, const int *__restrict__ selected,
                                  long long n, double *__restrict__ state, int nx_, int ny_, int nz_, double rho0,
                                  double ux, double uy, double uz) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int li = selected[i];
    const int x = L.x[li], y = L.y[li], z = L.z[li], d = L.d[li], di = inv(d);
    state[2 * i] = load_g(pdf, G, di, x + cx(d) - nx_, y + cy(d) - ny_, G.wrapz(z + cz(d) - nz_));
    const double u[3] = {ux, uy, uz};
    const int c[3] = {cx(di), cy(di), cz(di)};
    double p = rho0;
    for (int a = 0; a < 3; ++a) p *= c[a] == 0 ? 2.0 / 3.0 - u[a] * u[a] : 0.5 * (1.0 / 3.0 + u[a] * u[a] + c[a] * u[a]);
    state[2 * i + 1] = p - weight(di);
}

// characteristic farfield, farfield.py:144-206
struct FarfieldObject {
    int normal[3];
    int mode;            // 0 inflow (fixed invariant), 1 evolving outflow, 2 glancing
    double nh[3];        // unit normal
    double un_inf;       // n.U
    double ut_inf[3];    // U - un_inf n
    double P[3][3];      // I - n n^T
    int active[3];       // axes carrying a transverse term
    double density;
    double vel[3];
    // the same constants rounded to FP32, read by the FP32-arithmetic forms
    float nh_f[3], un_inf_f, ut_inf_f[3], P_f[3][3], density_f, vel_f[3];
};
// an object constant in the arithmetic type T
__device__ __forceinline__ double ffv(double d, float, double) { return d; }
__device__ __forceinline__ float ffv(double, float f, float) { return f; }
// the eight objects live in device memory (indexed per link at run time)
struct FarfieldParams {
    const FarfieldObject *obj;
    int nobj;
};

template <typename S>
__device__ __forceinline__ void macro_at(const S *pdf, const Grid &G, int x, int y, int z, double &rho, double u[3]) {
    double d = 0.0, j[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const double g = load_g(pdf, G, q, x, y, z);
        d += g;
        j[0] += cx(q) * g;
        j[1] += cy(q) * g;
        j[2] += cz(q) * g;
    }
    rho = 1.0 + d;
    for (int a = 0; a < 3; ++a) u[a] = j[a] / rho;
}

// density, velocity and ln(density) of one cell in the storage form's
// arithmetic type (FP64 for the plain form, FP32 for the others)
template <typename S>
__device__ __forceinline__ void macro_lr(const S *pdf, const Grid &G, int x, int y, int z,
                                         typename Store<S>::A &rho, typename Store<S>::A u[3],
                                         typename Store<S>::A &lr) {
    using T = typename Store<S>::A;
    if constexpr (sizeof(T) == 8) {
        macro_at(pdf, G, x, y, z, rho, u);
        lr = log(rho);
    } else {
        T d = 0, j[3] = {0, 0, 0};
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const T g = Store<S>::load(pdf + q * G.qs + G.cell(x, y, z), q, G.shift[q]);
            d += g;
            if (cx(q)) j[0] += cx(q) > 0 ? g : -g;
            if (cy(q)) j[1] += cy(q) > 0 ? g : -g;
            if (cz(q)) j[2] += cz(q) > 0 ? g : -g;
        }
        rho = T(1) + d;
        for (int a = 0; a < 3; ++a) u[a] = j[a] / rho;
        lr = log1pf(d);
    }
}

// The farfield reads density, velocity and ln(rho) of the fluid cells next to
// the ghost ring only (the feet of its links and their neighbours along the
// boundary).  They are computed once per step for that one-cell-wide band
// ("ring": interior cells with x in {0, nx-1} or y in {0, ny-1}) and looked up
// by the links, instead of being recomputed by every link that touches them.
struct alignas(32) Macro4 {
    double rho, ux, uy, uz;
};
struct Ring {
    Macro4 *ru;   // (rho, ux, uy, uz) per z and ring cell (float4 in the FP32 forms)
    double *lr;   // ln(rho) (float in the FP32 forms)
    long long n;  // ring cells per z-plane: 2 nx + 2 (ny - 2)
};
template <typename T>
__device__ __forceinline__ void ring_put(const Ring &R, long long i, T rho, const T u[3], T lr) {
    if constexpr (sizeof(T) == 8) {
        R.ru[i] = Macro4{rho, u[0], u[1], u[2]};
        R.lr[i] = lr;
    } else {
        reinterpret_cast<float4 *>(R.ru)[i] = make_float4(rho, u[0], u[1], u[2]);
        reinterpret_cast<float *>(R.lr)[i] = lr;
    }
}
__device__ __forceinline__ long long ring_index(const Grid &G, int x, int y) {  // interior coordinates
    if (y == 0) return x;
    if (y == G.ny - 1) return G.nx + x;
    if (x == 0) return 2LL * G.nx + (y - 1);
    return 2LL * G.nx + (G.ny - 2) + (y - 1);  // x == nx - 1
}
__device__ __forceinline__ void ring_cell(const Grid &G, long long r, int &x, int &y) {
    if (r < G.nx) { x = (int)r; y = 0; return; }
    if (r < 2LL * G.nx) { x = (int)(r - G.nx); y = G.ny - 1; return; }
    const long long k = r - 2LL * G.nx;
    if (k < G.ny - 2) { x = 0; y = (int)k + 1; return; }
    x = G.nx - 1;
    y = (int)(k - (G.ny - 2)) + 1;
}

template <typename S>
__device__ __forceinline__ void ring_macro_item(const S *__restrict__ pdf, const Grid &G, const Ring &R, long long i) {
    using T = typename Store<S>::A;
    const int z = (int)(i / R.n);
    const long long r = i - (long long)z * R.n;
    int x, y;
    ring_cell(G, r, x, y);
    T rho, u[3], lr;
    macro_lr(pdf, G, x + 1, y + 1, z, rho, u, lr);
    ring_put(R, i, rho, u, lr);
}

template <typename S>
__global__ void k_ring_macros(const S *__restrict__ pdf, Grid G, Ring R) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= R.n * G.nz) return;
    ring_macro_item(pdf, G, R, i);
}

template <typename T>
__device__ __forceinline__ void ring_get(const Grid &G, const Ring &R, int px, int py, int z, T &rho, T u[3],
                                         T &lr) {  // padded x, y
    const long long i = (long long)z * R.n + ring_index(G, px - 1, py - 1);
    if constexpr (sizeof(T) == 8) {
        const Macro4 v = R.ru[i];
        rho = v.rho;
        u[0] = v.ux;
        u[1] = v.uy;
        u[2] = v.uz;
        lr = R.lr[i];
    } else {
        const float4 v = reinterpret_cast<const float4 *>(R.ru)[i];
        rho = v.x;
        u[0] = v.y;
        u[1] = v.z;
        u[2] = v.w;
        lr = reinterpret_cast<const float *>(R.lr)[i];
    }
}

// transverse term F of the evolving outflow invariant (farfield.py:162-180)
template <typename T>
__device__ T farfield_transverse(const Grid &G, const Ring &R, const FarfieldObject &o, const int foot[3],
                                 const signed char edge[3], const T u[3], T rm) {
    T F = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (!o.active[a]) continue;
        const int e = edge[a];
        const int off1 = e == -1 ? 1 : -1;
        const int off2 = e == 0 ? 1 : -2 * e;
        const T c0 = T(1.5) * e;
        const T c1 = e == 0 ? T(-0.5) : T(-2.0) * e;
        const T c2 = e == 0 ? T(0.5) : T(0.5) * e;
        int s1[3] = {foot[0], foot[1], foot[2]}, s2[3] = {foot[0], foot[1], foot[2]};
        s1[a] += off1;
        s2[a] += off2;
        s1[2] = G.wrapz(s1[2]);
        s2[2] = G.wrapz(s2[2]);
        T r1, v1[3], l1, r2, v2[3], l2;
        ring_get(G, R, s1[0], s1[1], s1[2], r1, v1, l1);
        ring_get(G, R, s2[0], s2[1], s2[2], r2, v2, l2);
        T du[3];
        for (int b = 0; b < 3; ++b) du[b] = c0 * u[b] + c1 * v1[b] + c2 * v2[b];
        // ln(rho / density) with density 1 for every object
        const T nh[3] = {ffv(o.nh[0], o.nh_f[0], T(0)), ffv(o.nh[1], o.nh_f[1], T(0)), ffv(o.nh[2], o.nh_f[2], T(0))};
        const T rm1 = nh[0] * v1[0] + nh[1] * v1[1] + nh[2] * v1[2] - T(CS) * l1;
        const T rm2 = nh[0] * v2[0] + nh[1] * v2[1] + nh[2] * v2[2] - T(CS) * l2;
        F += ffv(o.un_inf, o.un_inf_f, T(0)) * (ffv(o.P[a][0], o.P_f[a][0], T(0)) * du[0] + ffv(o.P[a][1], o.P_f[a][1], T(0)) * du[1] + ffv(o.P[a][2], o.P_f[a][2], T(0)) * du[2]) -
             ffv(o.ut_inf[a], o.ut_inf_f[a], T(0)) * (c0 * rm + c1 * rm1 + c2 * rm2);
    }
    return F;
}

template <typename T>
__device__ __forceinline__ T feq_dir(T r, const T v[3], int q) {
    const int c[3] = {cx(q), cy(q), cz(q)};
    T p = r;
    for (int a = 0; a < 3; ++a) {
        const T cc = (T)c[a], w = v[a];
        p *= T(2.0 / 3.0) - w * w + (T(1.5) * w * w - T(0.5)) * cc * cc + cc * w / T(2.0);
    }
    return p;
}

template <typename S>
__device__ __forceinline__ void farfield_link(S *__restrict__ pdf, const Grid &G, const OuterLinks &L,
                                              const FarfieldParams &P, const Ring &R, double *__restrict__ incoming,
                                              double *__restrict__ derivative, long long *__restrict__ clock,
                                              const double *__restrict__ init_lo, const double *__restrict__ init_hi,
                                              int prepare, long long i) {
    using T = typename Store<S>::A;
    const int x = L.x[i], y = L.y[i], z = L.z[i], d = L.d[i], di = inv(d);
#ifdef AK_CHECKED
    if (L.obj[i] < 0 || L.obj[i] >= P.nobj) {
        AK_CHECK(G, -1, x, y, z, 4);
        return;
    }
#endif
    const FarfieldObject &o = P.obj[L.obj[i]];
    // foot = x + c_d - n: a fluid cell next to the ghost cell, wrapped in z
    const int foot[3] = {x + cx(d) - o.normal[0], y + cy(d) - o.normal[1], G.wrapz(z + cz(d) - o.normal[2])};
    const signed char edge[3] = {L.edge[2 * i], L.edge[2 * i + 1], 0};
    T rho, u[3], lr;
    ring_get(G, R, foot[0], foot[1], foot[2], rho, u, lr);
    const T nh[3] = {ffv(o.nh[0], o.nh_f[0], T(0)), ffv(o.nh[1], o.nh_f[1], T(0)), ffv(o.nh[2], o.nh_f[2], T(0))};
    const T un_inf = ffv(o.un_inf, o.un_inf_f, T(0));
    const T un = nh[0] * u[0] + nh[1] * u[1] + nh[2] * u[2];
    const T rm = un - T(CS) * lr, rp = un + T(CS) * lr;
    if (prepare) {
        // farfield.py:84-113: seed the trapezoid so the first update returns
        // the actual initial invariant
        if (o.mode == 1) {
            const T F = farfield_transverse(G, R, o, foot, edge, u, rm);
            incoming[i] = rm - F;
            derivative[i] = F;
        } else if (o.mode == 2) {
            clock[i] = 0;
        } else {
            incoming[i] = o.un_inf;
            derivative[i] = 0.0;
        }
        return;
    }
    T value, F = 0;
    if (o.mode == 1) {
        F = farfield_transverse(G, R, o, foot, edge, u, rm);
        value = T(incoming[i]) + (F + T(derivative[i])) / T(2.0);
    } else if (o.mode == 2) {
        // one linear interpolation of the saved initial invariant at the shift
        // U * clock along x (the only axis with U != 0), zero outside
        const double target = (double)(foot[0] - 1) - o.vel[0] * (double)clock[i];
        const int lower = (int)floor(target);
        const T frac = T(target - lower);
        const double *row = o.normal[1] < 0 ? init_lo : init_hi;
        T sum = 0;
        for (int bit = 0; bit < 2; ++bit) {
            const int k = lower + bit;
            const T w = bit ? frac : T(1) - frac;
            const int kc = k < 0 ? 0 : (k > G.nx - 1 ? G.nx - 1 : k);
            const T sample = T(row[(long long)kc * G.nz + foot[2]]);
            sum += w * ((k >= 0 && k < G.nx) ? sample : T(0));
        }
        value = un_inf + sum;
    } else {
        value = un_inf;
    }
    const T unb = (rp + value) / T(2.0);
    const T rhob = ffv(o.density, o.density_f, T(0)) * exp((rp - value) / (T(2.0) * T(CS)));
    T ub[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const T tangential = unb >= T(0) ? u[a] - nh[a] * un : ffv(o.vel[a], o.vel_f[a], T(0)) - nh[a] * un_inf;
        ub[a] = nh[a] * unb + tangential;
    }
    const T foot_g = (T)Store<S>::load(pdf + di * G.qs + G.cell(foot[0], foot[1], foot[2]), di, G.shift[di]);
    const T ghost = foot_g + feq_dir(rhob, ub, di) - feq_dir(rho, u, di);
    store_g(pdf, G, di, x + cx(d), y + cy(d), G.wrapz(z + cz(d)), (double)ghost);
    if (o.mode == 1) {
        incoming[i] = value;
        derivative[i] = F;
    } else if (o.mode == 2) {
        clock[i] += 1;
    }
}

template <typename S>
__global__ void __launch_bounds__(256) k_farfield(S *__restrict__ pdf, Grid G, OuterLinks L, FarfieldParams P, Ring R,
                                                  double *__restrict__ incoming, double *__restrict__ derivative,
                                                  long long *__restrict__ clock, const double *__restrict__ init_lo,
                                                  const double *__restrict__ init_hi, int prepare) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= L.n) return;
    farfield_link(pdf, G, L, P, R, incoming, derivative, clock, init_lo, init_hi, prepare, i);
}

// glancing faces: initial invariant u.n - cs ln(rho/rho_inf) - un_inf on the
// fluid row next to the face (the only row the transport reads)
template <typename T>
__global__ void k_glancing_rows(Grid G, FarfieldParams P, Ring R, double *__restrict__ lo, double *__restrict__ hi) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)G.nx * G.nz) return;
    const int x = (int)(i / G.nz) + 1, z = (int)(i - (i / G.nz) * G.nz);
    for (int k = 0; k < P.nobj; ++k) {
        const FarfieldObject &o = P.obj[k];
        if (o.mode != 2) continue;
        const int y = o.normal[1] < 0 ? 1 : G.ny;
        T rho, u[3], lr;
        ring_get(G, R, x, y, z, rho, u, lr);
        const T v = ffv(o.nh[0], o.nh_f[0], T(0)) * u[0] + ffv(o.nh[1], o.nh_f[1], T(0)) * u[1] + ffv(o.nh[2], o.nh_f[2], T(0)) * u[2] - T(CS) * lr - ffv(o.un_inf, o.un_inf_f, T(0));
        (o.normal[1] < 0 ? lo : hi)[i] = v;
    }
}

// ------------------------------------------------------------ fields
__device__ __forceinline__ void equilibrium_g(double rho, const double u[3], double g[Q]) {
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int c[3] = {cx(q), cy(q), cz(q)};
        double p = rho;
        for (int a = 0; a < 3; ++a)
            p *= c[a] == 0 ? 2.0 / 3.0 - u[a] * u[a] : 0.5 * (1.0 / 3.0 + u[a] * u[a] + c[a] * u[a]);
        g[q] = p - weight(q);
    }
}

// solver.py:157-202 on the device: freestream plus the divergence-free seed
template <typename S>
__global__ void k_init_perturbed(S *__restrict__ pdf, Grid G, const uint8_t *__restrict__ flags, double speed,
                                 double amp, double phase_y, double phase_z, double lead_x, double lead_y,
                                 double origin_x, double origin_y, double dx, double ky, double kz) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)G.nx * G.ny * G.nz) return;
    const int z = (int)(i % G.nz);
    const long long xy = i / G.nz;
    const int y = (int)(xy % G.ny), x = (int)(xy / G.ny);
    double u[3] = {speed, 0.0, 0.0};
    const double xm = x + 0.5, ym = y + 0.5, zm = z + 0.5;
    const double rel_x = (xm * dx + origin_x) - lead_x, rel_y = (ym * dx + origin_y) - lead_y;
    const double zz = zm * dx;
    const double t = (rel_x - 0.5) / 0.75;
    const double env = exp(-(t * t));
    u[1] = amp * sin(ky * rel_y + phase_y) * cos(kz * zz + phase_z) * env;
    u[2] = -amp * ky / kz * cos(ky * rel_y + phase_y) * sin(kz * zz + phase_z) * env;
    if (flags[(y + 1) * G.nxp + (x + 1)] != FLAG_FLUID) u[0] = u[1] = u[2] = 0.0;
    double g[Q];
    equilibrium_g(1.0, u, g);
    for (int q = 0; q < Q; ++q) store_g(pdf, G, q, x + 1, y + 1, z, g[q]);
}

// rho/u given per interior cell in (x, y, z) order
template <typename S>
__global__ void k_init_fields(S *__restrict__ pdf, Grid G, const double *__restrict__ rho,
                              const double *__restrict__ vel) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)G.nx * G.ny * G.nz) return;
    const int z = (int)(i % G.nz);
    const long long xy = i / G.nz;
    const int y = (int)(xy % G.ny), x = (int)(xy / G.ny);
    const double u[3] = {vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]};
    double g[Q];
    equilibrium_g(rho[i], u, g);
    for (int q = 0; q < Q; ++q) store_g(pdf, G, q, x + 1, y + 1, z, g[q]);
}

// (x, y, z, 27) doubles <-> device layout
template <typename S>
__global__ void k_export(const S *__restrict__ pdf, Grid G, double *__restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)G.nx * G.ny * G.nz) return;
    const int z = (int)(i % G.nz);
    const long long xy = i / G.nz;
    const int y = (int)(xy % G.ny), x = (int)(xy / G.ny);
    for (int q = 0; q < Q; ++q) out[i * Q + q] = load_g(pdf, G, q, x + 1, y + 1, z);
}
template <typename S>
__global__ void k_import(S *__restrict__ pdf, Grid G, const double *__restrict__ in) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)G.nx * G.ny * G.nz) return;
    const int z = (int)(i % G.nz);
    const long long xy = i / G.nz;
    const int y = (int)(xy % G.ny), x = (int)(xy / G.ny);
    for (int q = 0; q < Q; ++q) store_g(pdf, G, q, x + 1, y + 1, z, in[i * Q + q]);
}

template <typename S>
__global__ void k_macros(const S *__restrict__ pdf, Grid G, double *__restrict__ rho, double *__restrict__ vel) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)G.nx * G.ny * G.nz) return;
    const int z = (int)(i % G.nz);
    const long long xy = i / G.nz;
    const int y = (int)(xy % G.ny), x = (int)(xy / G.ny);
    double r, u[3];
    macro_at(pdf, G, x + 1, y + 1, z, r, u);
    rho[i] = r;
    vel[3 * i] = u[0];
    vel[3 * i + 1] = u[1];
    vel[3 * i + 2] = u[2];
}

// validity reduction over fluid cells (solver.py:281-297):
// partial[block] = (max |u|^2, max |rho-1|, min rho (as -max -rho), sum rho, count non-finite)
template <typename S>
__global__ void __launch_bounds__(256) k_diagnostics(const S *__restrict__ pdf, Grid G,
                                                     const uint8_t *__restrict__ flags, double *__restrict__ partials) {
    const long long n = (long long)G.nx * G.ny * G.nz;
    double mx_u2 = 0.0, mx_dr = 0.0, mx_neg = -1e300, sum = 0.0, bad = 0.0, cnt = 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % G.nx);
        const long long yz = i / G.nx;
        const int y = (int)(yz % G.ny), z = (int)(yz / G.ny);
        if (flags[(y + 1) * G.nxp + (x + 1)] != FLAG_FLUID) continue;
        double r, u[3];
        macro_at(pdf, G, x + 1, y + 1, z, r, u);
        const double u2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
        if (!isfinite(r) || !isfinite(u2)) {
            bad += 1.0;
            continue;
        }
        mx_u2 = fmax(mx_u2, u2);
        mx_dr = fmax(mx_dr, fabs(r - 1.0));
        mx_neg = fmax(mx_neg, -r);
        sum += r;
        cnt += 1.0;
    }
    __shared__ double red[32][6];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        mx_u2 = fmax(mx_u2, __shfl_down_sync(0xffffffffu, mx_u2, o));
        mx_dr = fmax(mx_dr, __shfl_down_sync(0xffffffffu, mx_dr, o));
        mx_neg = fmax(mx_neg, __shfl_down_sync(0xffffffffu, mx_neg, o));
        sum += __shfl_down_sync(0xffffffffu, sum, o);
        bad += __shfl_down_sync(0xffffffffu, bad, o);
        cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    }
    if (lane == 0) {
        red[warp][0] = mx_u2;
        red[warp][1] = mx_dr;
        red[warp][2] = mx_neg;
        red[warp][3] = sum;
        red[warp][4] = bad;
        red[warp][5] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = blockDim.x >> 5;
        double a[6] = {red[0][0], red[0][1], red[0][2], red[0][3], red[0][4], red[0][5]};
        for (int w = 1; w < nw; ++w) {
            a[0] = fmax(a[0], red[w][0]);
            a[1] = fmax(a[1], red[w][1]);
            a[2] = fmax(a[2], red[w][2]);
            a[3] += red[w][3];
            a[4] += red[w][4];
            a[5] += red[w][5];
        }
        for (int k = 0; k < 6; ++k) partials[blockIdx.x * 6 + k] = a[k];
    }
}

// Reduction of nrows rows of NV partial values (column k a maximum when bit k
// of max_mask is set, else a sum) by one block of REDUCE_THREADS threads: a
// fixed strided accumulation, then a fixed shared-memory tree, so the result
// does not depend on scheduling.  Thread 0 returns the reduced row.
constexpr int REDUCE_THREADS = 256;
// the block's fixed-order tree over every thread's acc (maxima where
// max_mask has the bit, sums elsewhere); the result in every thread's acc
template <int NV>
__device__ void reduce_block(unsigned max_mask, double (&acc)[NV]);
template <int NV>
__device__ void reduce_rows(const double *__restrict__ rows, long long nrows, unsigned max_mask, double (&acc)[NV]) {
    const int t = threadIdx.x;
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = ((max_mask >> k) & 1) ? -INFINITY : 0.0;
    for (long long b = t; b < nrows; b += REDUCE_THREADS)
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const double v = rows[b * NV + k];
            acc[k] = ((max_mask >> k) & 1) ? fmax(acc[k], v) : acc[k] + v;
        }
    reduce_block<NV>(max_mask, acc);
}
template <int NV>
__device__ void reduce_block(unsigned max_mask, double (&acc)[NV]) {
    __shared__ double red[NV][REDUCE_THREADS];
    const int t = threadIdx.x;
#pragma unroll
    for (int k = 0; k < NV; ++k) red[k][t] = acc[k];
    __syncthreads();
    for (int stride = REDUCE_THREADS / 2; stride > 0; stride >>= 1) {
        if (t < stride)
#pragma unroll
            for (int k = 0; k < NV; ++k)
                red[k][t] = ((max_mask >> k) & 1) ? fmax(red[k][t], red[k][t + stride]) : red[k][t] + red[k][t + stride];
        __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = red[k][0];
}

__global__ void __launch_bounds__(REDUCE_THREADS)
    k_diagnostics_final(const double *__restrict__ partials, int nblocks, double *__restrict__ out) {
    double a[6];
    reduce_rows<6>(partials, nblocks, 0x7u, a);
    if (threadIdx.x == 0)
        for (int k = 0; k < 6; ++k) out[k] = a[k];
}

}  // namespace ak
