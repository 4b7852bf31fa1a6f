// ak_batch.cuh -- many independent uniform cases advanced by one set of
// launches per step.
//
// A batch holds a device array of per-case descriptors (BatchCase) and, for
// every kernel of the uniform step, a packed work table of (case, chunk)
// items: the characteristic farfield's ring macros and links, the legacy
// boundary's UBB cells and outflow links, the Bouzidi wall links and the
// fused stream-collide blocks.  A step is therefore four to six launches
// (one more when loads are sampled) whatever the number of cases, each
// kernel running the same per-item body as the single-case kernel
// (ak_kernels.cuh) on the item's case, so a case computes the same bits alone
// and in any mix.  The stream-collide launch is persistent: a fixed grid of
// CTAs strides over the packed block table, whose block width, grid size and
// ordering (case-major or interleaved) the host tunes per batch.
#pragma once
#include "ak_kernels.cuh"

namespace ak {

template <typename S>
struct BatchCase {
    S *pdf[2];
    const uint8_t *flags;
    Grid G;
    typename Store<S>::T omega_s, omega_b;
    Sgs<typename Store<S>::T> sgs;  // Smagorinsky constants (c18 = 0: molecular viscosity)
    int cur0;  // copy holding the case's state at batch parity 0
    int n_elements;
    double ox, oy;
    // legacy outer boundary (UBB cells, outflow links and their history)
    const int *ubb_cells;
    long long n_ubb_cells;
    double speed;
    const int *sel_out;
    long long n_out;
    double *out_state;
    // characteristic farfield
    OuterLinks L;
    FarfieldParams P;
    Ring R;
    double *ff_in, *ff_der;
    long long *ff_clock;
    const double *ff_lo, *ff_hi;
    // Bouzidi walls and their load partials [element][block][5]
    const WallKey *keys;
    const double *wall_q;
    long long nkeys;
    double *partials;
    long long wall_blocks;
};

struct WorkItem {
    int c;      // case
    int chunk;  // block of that case's items
};

template <typename S>
__device__ __forceinline__ S *batch_src(const BatchCase<S> &c, int parity) {
    return c.pdf[c.cur0 ^ parity];
}

template <typename S>
__global__ void __launch_bounds__(256)
    k_batch_ring_macros(const BatchCase<S> *__restrict__ cases, const WorkItem *__restrict__ work, int parity) {
    const WorkItem w = work[blockIdx.x];
    const BatchCase<S> &c = cases[w.c];
    const long long i = (long long)w.chunk * blockDim.x + threadIdx.x;
    if (i >= c.R.n * c.G.nz) return;
    ring_macro_item(batch_src(c, parity), c.G, c.R, i);
}

template <typename S>
__global__ void __launch_bounds__(256)
    k_batch_farfield(const BatchCase<S> *__restrict__ cases, const WorkItem *__restrict__ work, int parity) {
    const WorkItem w = work[blockIdx.x];
    const BatchCase<S> &c = cases[w.c];
    const long long i = (long long)w.chunk * blockDim.x + threadIdx.x;
    if (i >= c.L.n) return;
    farfield_link(batch_src(c, parity), c.G, c.L, c.P, c.R, c.ff_in, c.ff_der, c.ff_clock, c.ff_lo, c.ff_hi, 0, i);
}

// legacy outer boundary: UBB (solver.py:131) then the ExtrapolationOutflow,
// in the single-case step's order
template <typename S>
__global__ void __launch_bounds__(256)
    k_batch_ubb(const BatchCase<S> *__restrict__ cases, const WorkItem *__restrict__ work, int parity) {
    const WorkItem w = work[blockIdx.x];
    const BatchCase<S> &c = cases[w.c];
    const long long i = (long long)w.chunk * blockDim.x + threadIdx.x;
    if (i >= c.n_ubb_cells * c.G.nz) return;
    ubb_item(batch_src(c, parity), c.G, c.ubb_cells, c.n_ubb_cells, c.speed, 0.0, 0.0, i);
}

template <typename S>
__global__ void __launch_bounds__(256)
    k_batch_outflow(const BatchCase<S> *__restrict__ cases, const WorkItem *__restrict__ work, int parity) {
    const WorkItem w = work[blockIdx.x];
    const BatchCase<S> &c = cases[w.c];
    const long long i = (long long)w.chunk * blockDim.x + threadIdx.x;
    if (i >= c.n_out) return;
    outflow_item(batch_src(c, parity), c.G, c.L, c.sel_out, c.out_state, 1, 0, 0, i);
}

template <typename S>
__global__ void __launch_bounds__(256) k_batch_walls(const BatchCase<S> *__restrict__ cases,
                                                     const WorkItem *__restrict__ work, int parity, int sample) {
    const WorkItem w = work[blockIdx.x];
    const BatchCase<S> &c = cases[w.c];
    const long long tid = (long long)w.chunk * blockDim.x + threadIdx.x;
    double acc[5] = {0, 0, 0, 0, 0};
    int element = -1;
    if (tid < c.nkeys * c.G.nz * 3) wall_link(batch_src(c, parity), c.G, c.keys, c.wall_q, tid, sample, c.ox, c.oy, acc, element);
    if (!sample) return;
    wall_block_sums(acc, element, c.n_elements, c.partials, w.chunk, c.wall_blocks);
}

// loads[case][MAX_ELEMENTS * 5]: the per-element sums of k_sum_partials, in
// the same lane-strided order
template <typename S>
__global__ void k_batch_sum_partials(const BatchCase<S> *__restrict__ cases, double *__restrict__ loads) {
    const BatchCase<S> &c = cases[blockIdx.y];
    const int t = blockIdx.x, lane = threadIdx.x;
    if (t >= 5 * c.n_elements) return;
    const int e = t / 5, k = t - 5 * (t / 5);
    double s = 0.0;
    for (long long b = lane; b < c.wall_blocks; b += 32) s += c.partials[((long long)e * c.wall_blocks + b) * 5 + k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) loads[(long long)blockIdx.y * 5 * MAX_ELEMENTS + t] = s;
}

// fused pull-stream + collision over the packed block table: block chunk of
// a case covers its stream-collide items [chunk * TB, chunk * TB + TB) in
// the single-case kernel's numbering (cells across rows, or cell pairs in
// the pair forms), so a case's bits do not depend on the batch and no warp
// is left part-empty at a row's end.  The pair forms take one table entry
// per block (the grid is the table): the state of a persistent loop over the
// table, held across the collision, made the FP16 body spill at five
// resident blocks; the other forms loop over the table on a persistent grid.
// resident 128-thread blocks per SM: the pair forms' body also holds the
// case descriptor, and spills at the single-case FP16 kernel's six blocks
// (80 registers); the FP16 form runs at five (96 registers, no spill), the
// FP32 form at four
template <typename S>
__host__ __device__ constexpr int batch_bulk_min_blocks() {
    return pair_form<S>() ? (std::is_same_v<S, __half> ? 5 : 4) : Store<S>::MIN_BLOCKS;
}
template <typename S, int TB>
__global__ void __launch_bounds__(TB, batch_bulk_min_blocks<S>() * 128 / TB)
    k_batch_bulk(const BatchCase<S> *__restrict__ cases, const WorkItem *__restrict__ work, long long n_work,
                 int parity) {
    if constexpr (pair_form<S>()) {
        if ((long long)blockIdx.x >= n_work) return;
        const WorkItem w = work[blockIdx.x];
        const BatchCase<S> &c = cases[w.c];
        const Grid &G = c.G;
        const int4 none = make_int4(0, 0, 0, 0);
        stream_collide_pair_item(c.pdf[c.cur0 ^ parity], c.pdf[c.cur0 ^ parity ^ 1], c.flags, G, G.shift,
                                 c.omega_s, c.omega_b, c.sgs, none, make_int4(1, G.nx + 1, 1, G.ny + 1), none,
                                 (long long)w.chunk * TB + threadIdx.x);
    } else {
        for (long long e = blockIdx.x; e < n_work; e += gridDim.x) {
            const WorkItem w = work[e];
            const BatchCase<S> &c = cases[w.c];
            const Grid G = c.G;
            const long long i = (long long)w.chunk * TB + threadIdx.x;
            const S *src = c.pdf[c.cur0 ^ parity];
            S *dst = c.pdf[c.cur0 ^ parity ^ 1];
            const long long nxy = (long long)G.nx * G.ny;
            if (i >= nxy * G.nz) continue;
            const int z = (int)(i / nxy);
            const long long r = i - (long long)z * nxy;
            const int y = (int)(r / G.nx) + 1, x = (int)(r - (long long)(y - 1) * G.nx) + 1;
            stream_collide_cell(src, dst, c.flags, G, G.shift, c.omega_s, c.omega_b, x, y, z, c.sgs);
        }
    }
}

}  // namespace ak
