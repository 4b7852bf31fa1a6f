// ak_engine.cu -- host side of the C ABI declared in include/aerokinetic_gb300.h.
//
// Owns the device memory of each case, builds its boundary description on the
// GPU (flags, cut links, Bouzidi q) and on the host (the thin outer ring of
// links, O(surface)), and issues the per-step kernels on the case's stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/aerokinetic_gb300.h"
#include "ak_geometry.cuh"
#include "ak_transfer.cuh"
#include "ak_batch.cuh"
#include "ak_exterior.cuh"
#include "ak_peaks.cuh"

using namespace ak;

namespace {

thread_local std::string g_error;

int fail(int code, const std::string &msg) {
    g_error = msg;
    return code;
}

#define AK_CUDA(call)                                                                              \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return fail(e_ == cudaErrorMemoryAllocation ? AK_ERR_NOMEM : AK_ERR_CUDA,              \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                       \
    } while (0)

#define AK_TRY(call)              \
    do {                          \
        int r_ = (call);          \
        if (r_ != AK_OK) return r_; \
    } while (0)

long long blocks_for(long long n, int threads) { return (n + threads - 1) / threads; }

}  // namespace

namespace {
// grid of a stream-collide launch of 128-thread blocks over rect: one block
// per 128 items (cells, or cell pairs in the pair forms)
template <typename S>
unsigned stream_collide_grid(int4 rect, int nx, int ny, int nz) {
    return (unsigned)blocks_for(stream_collide_items<S>(rect, nx, ny, nz), 128);
}
// A launch with programmatic stream serialization: it may be scheduled while
// its predecessor on the stream drains (the launch latency of a chain of short
// kernels overlaps their tails); the kernel itself waits (chain_wait) before
// it touches memory.  Only kernels that start with chain_wait go through here.
// With chained false it is an ordinary launch.  A chained kernel's blocks
// can become resident while its predecessor still runs and then wait there,
// holding SM slots that concurrent branches (the far coarse pass, the other
// fine step) could use; the launch sites below are chained only where that
// measured faster (CHAIN_* flags).
template <typename... KArgs, typename... Args>
cudaError_t launch_chained(bool chained, void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t st,
                           Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = chained ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}
// which launch sites are chained: the fine steps' kernels after their donor
// moments' x pass (FINE), the x pass itself (PROLONG), the coarse
// transfer-block collision, near pass and donor moments (COARSE), the
// restriction, reflux and budget sums at the step's end (TAIL), the uniform
// step's bulk pass (UNIFORM).  Measured on the two-level benchmark case,
// graph-replayed ms per coarse step (FP32 / FP16 with FP32 walls / df64):
// none 0.1744 / 0.1649 / 0.496; FINE 0.1633 / 0.1528 / 0.495; FINE + PROLONG
// 0.1628 / 0.1527 / 0.495; + TAIL 0.1644 / 0.1539 / 0.494; all 0.1650 /
// 0.1553 / 0.483.  The FP64 step (1.107 ms) and the uniform steps do not move.
// coarse steps replayed per captured graph where the far pass runs on its own
// branch (1, 2 or 4): consecutive steps of one graph overlap the next step's
// start with the previous step's far pass
constexpr int STEPS_PER_GRAPH = 4;
constexpr bool CHAIN_FINE = true, CHAIN_PROLONG = true, CHAIN_COARSE = false, CHAIN_TAIL = false,
               CHAIN_UNIFORM = false;

// fixed grid of the per-case reductions whose results must not depend on the device
constexpr int STATS_BLOCKS_CASE = 4 * 152;

}  // namespace

struct ak_case {
    // description
    int nx = 0, ny = 0, nz = 0;
    double origin_x = 0, origin_y = 0, dx = 0, omega_s = 0, omega_b = 1, speed = 0;
    double smagorinsky = 0;  // subgrid constant C of the bulk collision (0: molecular viscosity)
    double ox = 0, oy = 0;  // origin / dx, the lever-arm offset of solver.py:239-240
    int farfield = 0, storage = 0, n_elements = 0;
    std::vector<int> poly_start, poly_count;
    std::vector<double> poly_xy;
    Grid G{};
    size_t esize = 8;
    // device memory
    void *pdf[2] = {nullptr, nullptr};
    int cur = 0;
    uint8_t *flags = nullptr;
    double *d_poly = nullptr;
    int *d_start = nullptr, *d_count = nullptr;
    WallKey *keys = nullptr;
    double *wall_q = nullptr;
    long long nkeys = 0, fallback = 0;
    // outer ring
    int *ox_ = nullptr, *oy_ = nullptr, *oz_ = nullptr;
    signed char *od = nullptr, *oobj = nullptr, *oedge = nullptr;
    long long nouter = 0;
    int *sel_ubb = nullptr, *sel_out = nullptr;
    long long n_ubb = 0, n_out = 0;
    int *ubb_cells = nullptr;  // (padded x, padded y, direction mask) per UBB cell
    long long n_ubb_cells = 0;
    double *out_state = nullptr;
    double *ff_in = nullptr, *ff_der = nullptr;
    long long *ff_clock = nullptr;
    double *ff_lo = nullptr, *ff_hi = nullptr;
    Macro4 *ring_ru = nullptr;
    double *ring_lr = nullptr;
    long long ring_n = 0;
    Ring ring() const { return Ring{ring_ru, ring_lr, ring_n}; }
    FarfieldObject ff_host[8];
    int ff_count = 0;
    FarfieldObject *d_ff = nullptr;
    float *d_shift = nullptr;
    Shift27 shift_host{};
    FarfieldParams ff() const { return FarfieldParams{d_ff, ff_count}; }
    // reductions
    double *partials = nullptr, *reduced = nullptr;
    long long partial_doubles = 0;
    // staging for host transfers
    double *staging = nullptr;
    size_t staging_doubles = 0;
    long long fluid_cells = 0;
    long long steps = 0;
    long long launches = 0;  // kernels issued by stepping since creation
    long long pdf_writes = 0;  // population writes from outside the step (set_pdf, init)
    bool prepared = false;
    int device = 0;  // CUDA device current when the case was created
    // stationarity residuals: the owned region (interior coordinates, an
    // excluded rectangle) and the device snapshot of (rho, j / U) per cell
    int res_region[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    double *res_snapshot = nullptr, *res_partials = nullptr, *res_out = nullptr;
    bool periodic_xy = false;  // the padded fine block of a refined case wraps in x and y
    // exterior farfield: the ghost layer is the auxiliary ring; band states
    // (log rho, u) of the cells within two of the edge (current and next), the
    // predictor's three stages, the initial incoming invariant of the glancing
    // rows, the source partials and out[10] (source, wall mass, running sums)
    ExtGeom ext{};
    double *ext_band[2] = {nullptr, nullptr};
    int ext_cur = 0;
    double *ext_stage[3] = {nullptr, nullptr, nullptr};
    double *ext_inc0 = nullptr, *ext_partials = nullptr, *ext_out = nullptr;
    long long ext_blocks = 0, wall_blocks = 0;
    // optional per-kernel timing: events recorded around each kernel group
    std::vector<cudaEvent_t> *timing = nullptr;
    cudaStream_t stream = nullptr;
    size_t device_bytes = 0;
    // ak_step replays the step from CUDA graphs, one per (copy parity,
    // sample), with the walls on a side stream beside the outer boundary; a
    // graph is captured again when the loads' partial sums have moved
    cudaGraphExec_t step_graph[4] = {nullptr, nullptr, nullptr, nullptr};
    double *graph_partials[4] = {nullptr, nullptr, nullptr, nullptr};
    long long graph_launches[4] = {0, 0, 0, 0};
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;

    OuterLinks outer() const { return OuterLinks{ox_, oy_, oz_, od, oobj, oedge, nouter}; }
};

namespace {

template <typename T>
int dalloc(ak_case *c, T **p, size_t count) {
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
    if (e != cudaSuccess)
        return fail(e == cudaErrorMemoryAllocation ? AK_ERR_NOMEM : AK_ERR_CUDA,
                    std::string("device allocation of ") + std::to_string(count * sizeof(T)) +
                        " bytes failed: " + cudaGetErrorString(e));
    c->device_bytes += count * sizeof(T);
    return AK_OK;
}

template <typename T>
int upload(ak_case *c, T **p, const std::vector<T> &v) {
    AK_TRY(dalloc(c, p, v.size()));
    if (!v.empty()) AK_CUDA(cudaMemcpyAsync(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, c->stream));
    return AK_OK;
}

void release(ak_case *c) {
    void *ptrs[] = {c->pdf[0], c->pdf[1], c->flags, c->d_poly, c->d_start, c->d_count, c->keys, c->wall_q,
                    c->ox_, c->oy_, c->oz_, c->od, c->oobj, c->oedge, c->sel_ubb, c->sel_out, c->out_state,
                    c->ubb_cells, c->ff_in, c->ff_der, c->ff_clock, c->ff_lo, c->ff_hi, c->partials, c->reduced,
                    c->staging, c->d_ff, c->d_shift, c->ring_ru, c->ring_lr, c->res_snapshot,
                    c->res_partials, c->res_out, c->ext_band[0], c->ext_band[1], c->ext_stage[0],
                    c->ext_stage[1], c->ext_stage[2], c->ext_inc0, c->ext_partials, c->ext_out};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (cudaGraphExec_t g : c->step_graph)
        if (g) cudaGraphExecDestroy(g);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->stream) cudaStreamDestroy(c->stream);
}

int ensure_staging(ak_case *c, size_t doubles) {
    if (c->staging_doubles >= doubles) return AK_OK;
    if (c->staging) {
        cudaFree(c->staging);
        c->device_bytes -= c->staging_doubles * sizeof(double);
        c->staging = nullptr;
    }
    AK_TRY(dalloc(c, &c->staging, doubles));
    c->staging_doubles = doubles;
    return AK_OK;
}

int ensure_partials(ak_case *c, long long doubles) {
    if (c->partial_doubles >= doubles) return AK_OK;
    if (c->partials) {
        cudaFree(c->partials);
        c->device_bytes -= c->partial_doubles * sizeof(double);
        c->partials = nullptr;
    }
    AK_TRY(dalloc(c, &c->partials, (size_t)doubles));
    c->partial_doubles = doubles;
    return AK_OK;
}

// ---- dispatch on the storage type
template <typename F>
int with_storage(ak_case *c, F &&f) {
    switch (c->storage) {
    case AK_STORAGE_F64: return f((double *)nullptr);
    case AK_STORAGE_F32: return f((float *)nullptr);
    case AK_STORAGE_F16: return f((__half *)nullptr);
    case AK_STORAGE_DF64: return f((df2 *)nullptr);
    }
    return fail(AK_ERR_INVALID, "unknown storage");
}

// ---- characteristic farfield objects, farfield.py:34-47 and 209-224
void build_farfield_objects(ak_case *c) {
    c->ff_count = 0;
    const double vel[3] = {c->speed, 0.0, 0.0};
    for (int nx_ = -1; nx_ <= 1; ++nx_)
        for (int ny_ = -1; ny_ <= 1; ++ny_) {
            if (nx_ == 0 && ny_ == 0) continue;
            FarfieldObject &o = c->ff_host[c->ff_count++];
            o.normal[0] = nx_;
            o.normal[1] = ny_;
            o.normal[2] = 0;
            const double len = std::sqrt((double)(nx_ * nx_ + ny_ * ny_));
            o.nh[0] = nx_ / len;
            o.nh[1] = ny_ / len;
            o.nh[2] = 0.0;
            o.density = 1.0;
            for (int a = 0; a < 3; ++a) o.vel[a] = vel[a];
            const double nu = nx_ * vel[0] + ny_ * vel[1];
            const bool any = vel[0] != 0 || vel[1] != 0 || vel[2] != 0;
            const bool evolve = nu >= 0 && any;
            const bool glancing = evolve && nu == 0;
            o.mode = glancing ? 2 : (evolve ? 1 : 0);
            o.un_inf = o.nh[0] * vel[0] + o.nh[1] * vel[1] + o.nh[2] * vel[2];
            for (int a = 0; a < 3; ++a) {
                o.ut_inf[a] = vel[a] - o.un_inf * o.nh[a];
                bool row = false;
                for (int b = 0; b < 3; ++b) {
                    o.P[a][b] = (a == b ? 1.0 : 0.0) - o.nh[a] * o.nh[b];
                    row |= o.P[a][b] != 0.0;
                }
                o.active[a] = !(o.ut_inf[a] == 0.0 && !row);
            }
            for (int a = 0; a < 3; ++a) {
                o.nh_f[a] = (float)o.nh[a];
                o.ut_inf_f[a] = (float)o.ut_inf[a];
                o.vel_f[a] = (float)o.vel[a];
                for (int b = 0; b < 3; ++b) o.P_f[a][b] = (float)o.P[a][b];
            }
            o.un_inf_f = (float)o.un_inf;
            o.density_f = (float)o.density;
        }
}

int farfield_object_of(const ak_case *c, int gx, int gy) {
    // ghost cell (gx, gy) in interior coordinates -> index of its normal in
    // the order built above
    const int nx_ = gx < 0 ? -1 : (gx >= c->nx ? 1 : 0);
    const int ny_ = gy < 0 ? -1 : (gy >= c->ny ? 1 : 0);
    for (int k = 0; k < c->ff_count; ++k)
        if (c->ff_host[k].normal[0] == nx_ && c->ff_host[k].normal[1] == ny_) return k;
    return -1;
}

// ---- outer ring links (pystencils index-list semantics: interior fluid cells
// with a neighbour in the ghost ring), built on the host: O(surface)
int build_outer(ak_case *c, const std::vector<uint8_t> &hflags) {
    std::vector<int> X, Y, Z;
    std::vector<signed char> D, OBJ, EDGE;
    std::vector<int> sel_ubb, sel_out;
    const int nx = c->nx, ny = c->ny, nz = c->nz, nxp = nx + 2;
    // boundary fluid cells face by face; links ordered (z, direction, cell) so
    // that consecutive links touch consecutive cells of a face (coalesced)
    std::vector<std::pair<int, int>> cells;  // interior coordinates
    auto add = [&](int x, int y) {
        if (hflags[(size_t)(y + 1) * nxp + (x + 1)] == FLAG_FLUID) cells.emplace_back(x, y);
    };
    for (int x = 0; x < nx; ++x) add(x, 0);
    if (ny > 1)
        for (int x = 0; x < nx; ++x) add(x, ny - 1);
    for (int y = 1; y < ny - 1; ++y) add(0, y);
    if (nx > 1)
        for (int y = 1; y < ny - 1; ++y) add(nx - 1, y);
    bool foot_outside = false;
    for (int z = 0; z < nz; ++z)
        for (int d = 1; d < Q; ++d)
            for (const auto &cell : cells) {
                const int x = cell.first, y = cell.second;
                const int gx = x + cx(d), gy = y + cy(d);
                if (gx >= 0 && gx < nx && gy >= 0 && gy < ny) continue;
                const long long idx = (long long)X.size();
                X.push_back(x + 1);
                Y.push_back(y + 1);
                Z.push_back(z);
                D.push_back((signed char)d);
                if (c->farfield == AK_FARFIELD_LEGACY) {
                    // UBB owns x<0, y<0, y>ny; the outflow (set later) owns x>nx
                    const bool outflow = gx >= nx;
                    OBJ.push_back(outflow ? 1 : 0);
                    (outflow ? sel_out : sel_ubb).push_back((int)idx);
                    EDGE.push_back(0);
                    EDGE.push_back(0);
                } else {
                    const int k = farfield_object_of(c, gx, gy);
                    OBJ.push_back((signed char)k);
                    const FarfieldObject &o = c->ff_host[k];
                    const int fx = x + cx(d) - o.normal[0], fy = y + cy(d) - o.normal[1];
                    foot_outside |= fx < 0 || fx >= nx || fy < 0 || fy >= ny;
                    EDGE.push_back((signed char)(fx == 0 ? -1 : (fx == nx - 1 ? 1 : 0)));
                    EDGE.push_back((signed char)(fy == 0 ? -1 : (fy == ny - 1 ? 1 : 0)));
                }
            }
    if (c->farfield == AK_FARFIELD_CHARACTERISTIC && foot_outside)
        return fail(AK_ERR_INVALID, "farfield foot cell outside the domain; the lattice is too small");
    c->nouter = (long long)X.size();
    AK_TRY(upload(c, &c->ox_, X));
    AK_TRY(upload(c, &c->oy_, Y));
    AK_TRY(upload(c, &c->oz_, Z));
    AK_TRY(upload(c, &c->od, D));
    AK_TRY(upload(c, &c->oobj, OBJ));
    AK_TRY(upload(c, &c->oedge, EDGE));
    if (c->farfield == AK_FARFIELD_LEGACY) {
        c->n_ubb = (long long)sel_ubb.size();
        c->n_out = (long long)sel_out.size();
        // the UBB links grouped by cell, face by face (coalesced along a face)
        std::vector<int> cells;
        auto ubb_cell = [&](int x, int y) {
            if (hflags[(size_t)(y + 1) * nxp + (x + 1)] != FLAG_FLUID) return;
            int mask = 0;
            for (int d = 1; d < Q; ++d) {
                const int gx = x + cx(d), gy = y + cy(d);
                if (gx >= 0 && gx < nx && gy >= 0 && gy < ny) continue;
                if (gx < nx) mask |= 1 << d;
            }
            if (!mask) return;
            cells.push_back(x + 1);
            cells.push_back(y + 1);
            cells.push_back(mask);
        };
        for (int x = 0; x < nx; ++x) ubb_cell(x, 0);
        if (ny > 1)
            for (int x = 0; x < nx; ++x) ubb_cell(x, ny - 1);
        for (int y = 1; y < ny - 1; ++y) ubb_cell(0, y);
        if (nx > 1)
            for (int y = 1; y < ny - 1; ++y) ubb_cell(nx - 1, y);
        c->n_ubb_cells = (long long)cells.size() / 3;
        AK_TRY(upload(c, &c->ubb_cells, cells));
        AK_TRY(upload(c, &c->sel_ubb, sel_ubb));
        AK_TRY(upload(c, &c->sel_out, sel_out));
        AK_TRY(dalloc(c, &c->out_state, (size_t)(2 * c->n_out)));
    } else {
        AK_TRY(upload(c, &c->d_ff, std::vector<FarfieldObject>(c->ff_host, c->ff_host + c->ff_count)));
        AK_TRY(dalloc(c, &c->ff_in, (size_t)c->nouter));
        AK_TRY(dalloc(c, &c->ff_der, (size_t)c->nouter));
        AK_TRY(dalloc(c, &c->ff_clock, (size_t)c->nouter));
        AK_TRY(dalloc(c, &c->ff_lo, (size_t)nx * nz));
        AK_TRY(dalloc(c, &c->ff_hi, (size_t)nx * nz));
        c->ring_n = 2LL * nx + 2LL * (ny - 2);
        AK_TRY(dalloc(c, &c->ring_ru, (size_t)(c->ring_n * nz)));
        AK_TRY(dalloc(c, &c->ring_lr, (size_t)(c->ring_n * nz)));
    }
    return AK_OK;
}

int build_geometry(ak_case *c, std::vector<uint8_t> &hflags) {
    const int nx = c->nx, ny = c->ny, nxp = nx + 2, nyp = ny + 2;
    AK_TRY(upload(c, &c->d_poly, c->poly_xy));
    AK_TRY(upload(c, &c->d_start, c->poly_start));
    AK_TRY(upload(c, &c->d_count, c->poly_count));
    Polygons P{c->d_poly, c->d_start, c->d_count, c->n_elements};
    AK_TRY(dalloc(c, &c->flags, (size_t)nxp * nyp));
    k_flags<<<dim3((unsigned)blocks_for(nxp, 128), nyp), 128, 0, c->stream>>>(c->flags, nx, ny, P, c->dx, c->origin_x,
                                                                               c->origin_y);
    AK_CUDA(cudaGetLastError());
    hflags.assign((size_t)nxp * nyp, 0);
    AK_CUDA(cudaMemcpyAsync(hflags.data(), c->flags, hflags.size(), cudaMemcpyDeviceToHost, c->stream));
    AK_CUDA(cudaStreamSynchronize(c->stream));
    std::vector<long long> per_element(c->n_elements, 0);
    long long fluid_columns = 0;
    for (int y = 0; y < nyp; ++y)
        for (int x = 0; x < nxp; ++x) {
            const uint8_t f = hflags[(size_t)y * nxp + x];
            const bool ghost = x == 0 || y == 0 || x == nx + 1 || y == ny + 1;
            if (ghost && f != FLAG_OUTER)
                return fail(AK_ERR_INVALID, "an element reaches the outer boundary; enlarge the domain");
            if (!ghost && f == FLAG_FLUID) ++fluid_columns;
            if (!ghost && f >= 1 && f <= c->n_elements) ++per_element[f - 1];
        }
    for (int e = 0; e < c->n_elements; ++e)
        if (per_element[e] == 0)
            return fail(AK_ERR_INVALID, "Element " + std::to_string(e) + " has no solid cells; increase resolution");
    c->fluid_cells = fluid_columns * c->nz;
    // compacted wall keys in (x, y, direction) order: every fluid column and
    // planar direction whose neighbour column is solid (pystencils index-list
    // semantics, deduplicated over z and c_z as solver.py:102-109 does)
    static const int planar[8] = {1, 2, 3, 4, 7, 8, 9, 10};
    std::vector<WallKey> keys;
    for (int x = 1; x <= nx; ++x)
        for (int y = 1; y <= ny; ++y) {
            if (hflags[(size_t)y * nxp + x] != FLAG_FLUID) continue;
            for (int k = 0; k < 8; ++k) {
                const int d = planar[k];
                const uint8_t nb = hflags[(size_t)(y + cy(d)) * nxp + x + cx(d)];
                if (nb >= 1 && nb <= c->n_elements) keys.push_back(WallKey{x, y, d, nb - 1});
            }
        }
    c->nkeys = (long long)keys.size();
    AK_TRY(upload(c, &c->keys, keys));
    AK_TRY(dalloc(c, &c->wall_q, (size_t)c->nkeys));
    int *status = nullptr;
    AK_TRY(dalloc(c, &status, (size_t)c->nkeys));
    if (c->nkeys) {
        k_wall_fractions<<<(unsigned)blocks_for(c->nkeys, 128), 128, 0, c->stream>>>(
            c->keys, c->nkeys, P, c->dx, c->origin_x, c->origin_y, c->wall_q, status);
        AK_CUDA(cudaGetLastError());
    }
    std::vector<int> hstatus((size_t)c->nkeys);
    std::vector<double> hq((size_t)c->nkeys);
    if (c->nkeys) {
        AK_CUDA(cudaMemcpyAsync(hstatus.data(), status, hstatus.size() * sizeof(int), cudaMemcpyDeviceToHost,
                                c->stream));
        AK_CUDA(cudaMemcpyAsync(hq.data(), c->wall_q, hq.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    }
    AK_CUDA(cudaStreamSynchronize(c->stream));
    cudaFree(status);
    c->device_bytes -= std::max<size_t>(1, (size_t)c->nkeys) * sizeof(int);
    c->fallback = 0;
    for (long long k = 0; k < c->nkeys; ++k) {
        if (hstatus[k]) return fail(AK_ERR_GEOMETRY, "A fluid-to-solid link has no geometric intersection");
        if (hq[k] == -1.0) c->fallback += 3LL * c->nz;
    }
    return AK_OK;
}

template <typename S>
int allocate_populations(ak_case *c) {
    const size_t n = (size_t)Q * c->G.qs;
    for (int k = 0; k < 2; ++k) {
        S *p = nullptr;
        AK_TRY(dalloc(c, &p, n));
        AK_CUDA(cudaMemsetAsync(p, 0, n * sizeof(S), c->stream));
        c->pdf[k] = p;
    }
    return AK_OK;
}

template <typename S>
S *src_of(ak_case *c) { return (S *)c->pdf[c->cur]; }
template <typename S>
S *dst_of(ak_case *c) { return (S *)c->pdf[1 - c->cur]; }

template <typename S>
int prepare_boundaries(ak_case *c) {
    S *src = src_of<S>(c);
    const int T = 256;
    if (c->farfield == AK_FARFIELD_LEGACY) {
        // the outflow state is seeded inside the first step, after the UBB
        // kernel (one_step): its corner links read ghost values the UBB writes
        c->prepared = true;
        return AK_OK;
    } else {
        k_ring_macros<S><<<(unsigned)blocks_for(c->ring_n * c->nz, T), T, 0, c->stream>>>(src, c->G, c->ring());
        AK_CUDA(cudaGetLastError());
        if (c->nouter) {
            k_farfield<S><<<(unsigned)blocks_for(c->nouter, T), T, 0, c->stream>>>(
                src, c->G, c->outer(), c->ff(), c->ring(), c->ff_in, c->ff_der, c->ff_clock, c->ff_lo, c->ff_hi, 1);
            AK_CUDA(cudaGetLastError());
        }
        k_glancing_rows<typename Store<S>::A><<<(unsigned)blocks_for((long long)c->nx * c->nz, T), T, 0, c->stream>>>(c->G, c->ff(), c->ring(),
                                                                                               c->ff_lo, c->ff_hi);
        AK_CUDA(cudaGetLastError());
    }
    c->prepared = true;
    return AK_OK;
}

void mark(ak_case *c) {
    if (!c->timing) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, c->stream);
    c->timing->push_back(e);
}

// the bulk collision's subgrid constants: tau0 = 1/omega and 18 C^2
template <typename S>
Sgs<typename Store<S>::T> sgs_of(const ak_case *c) {
    Sgs<typename Store<S>::T> m;
    if (c->smagorinsky > 0.0) {
        using R = typename SgsReal<typename Store<S>::T>::type;
        m.tau0 = R(1.0 / c->omega_s);
        m.c18 = R(18.0 * c->smagorinsky * c->smagorinsky);
    }
    return m;
}

template <typename S>
int exterior_step(ak_case *c, double *fixed_partials, long long fixed_capacity, bool branch);
constexpr int EXT_THREADS = 64;  // block width of the exterior ring kernels

// One step.  branch: the walls run on the case's side stream, forked before
// the outer boundary and joined before the bulk (the walls write only solid
// cells, the outer boundary only ghost cells, and each reads fluid cells the
// other does not write); used when the step is captured into a graph.
template <typename S>
int one_step(ak_case *c, bool sample, double *fixed_partials = nullptr, long long fixed_capacity = 0,
             bool branch = false) {
    using T = typename Store<S>::T;
    if (c->farfield == AK_FARFIELD_EXTERIOR) return exterior_step<S>(c, fixed_partials, fixed_capacity, branch);
    const bool first = !c->prepared;
    if (first) AK_TRY(prepare_boundaries<S>(c));
    S *src = src_of<S>(c);
    const int TB = 256;
    cudaStream_t ws = c->stream;
    if (branch) {
        AK_CUDA(cudaEventRecord(c->ev_fork, c->stream));
        AK_CUDA(cudaStreamWaitEvent(c->side, c->ev_fork, 0));
        ws = c->side;
    }
    mark(c);
    // outer boundary: the reference applies its boundary objects in
    // installation order; the outflow reads ghost values the UBB just wrote
    if (c->farfield == AK_FARFIELD_LEGACY) {
        if (c->n_ubb) {
            k_ubb<S><<<(unsigned)blocks_for(c->n_ubb_cells * c->nz, TB), TB, 0, c->stream>>>(
                src, c->G, c->ubb_cells, c->n_ubb_cells, c->speed, 0.0, 0.0);
            AK_CUDA(cudaGetLastError());
            ++c->launches;
        }
        if (c->n_out && first) {
            // ExtrapolationOutflow's initial history: the neighbour value as it
            // stands after the UBB of this step, matching the reference's
            // recorded legacy histories (docs/verification_farfield_20261107/
            // airfoil/legacy_down6) to 2e-13 over 960 steps
            k_outflow_prepare<S><<<(unsigned)blocks_for(c->n_out, TB), TB, 0, c->stream>>>(
                src, c->G, c->outer(), c->sel_out, c->n_out, c->out_state, 1, 0, 0, 1.0, c->speed, 0.0, 0.0);
            AK_CUDA(cudaGetLastError());
            ++c->launches;
        }
        if (c->n_out) {
            k_outflow<S><<<(unsigned)blocks_for(c->n_out, TB), TB, 0, c->stream>>>(src, c->G, c->outer(), c->sel_out,
                                                                                   c->n_out, c->out_state, 1, 0, 0);
            AK_CUDA(cudaGetLastError());
            ++c->launches;
        }
    } else if (c->nouter) {
        k_ring_macros<S><<<(unsigned)blocks_for(c->ring_n * c->nz, TB), TB, 0, c->stream>>>(src, c->G, c->ring());
        AK_CUDA(cudaGetLastError());
        k_farfield<S><<<(unsigned)blocks_for(c->nouter, TB), TB, 0, c->stream>>>(
            src, c->G, c->outer(), c->ff(), c->ring(), c->ff_in, c->ff_der, c->ff_clock, c->ff_lo, c->ff_hi, 0);
        AK_CUDA(cudaGetLastError());
        c->launches += 2;
    }
    mark(c);
    // walls and loads
    const long long nlinks = c->nkeys * c->nz * 3;
    if (nlinks) {
        const long long nb = blocks_for(nlinks, 256);
        double *partials = c->partials;
        if (sample && fixed_partials) {
            if (nb * 5 * c->n_elements > fixed_capacity)
                return fail(AK_ERR_INVALID, "wall links need " + std::to_string(nb * 5 * c->n_elements) +
                                                " partial sums; the static scratch holds " +
                                                std::to_string(fixed_capacity));
            partials = fixed_partials;
        } else if (sample) {
            AK_TRY(ensure_partials(c, nb * 5 * c->n_elements));
            partials = c->partials;
        }
        k_walls<S><<<(unsigned)nb, 256, 0, ws>>>(src, c->G, c->keys, c->wall_q, c->nkeys, sample ? 1 : 0,
                                                 c->n_elements, c->ox, c->oy, partials);
        AK_CUDA(cudaGetLastError());
        ++c->launches;
        if (sample) {
            k_sum_partials<<<5 * c->n_elements, 32, 0, ws>>>(partials, (int)nb, 5 * c->n_elements, c->reduced);
            AK_CUDA(cudaGetLastError());
            ++c->launches;
        }
    } else if (sample) {
        AK_CUDA(cudaMemsetAsync(c->reduced, 0, sizeof(double) * 5 * c->n_elements, ws));
    }
    if (branch) {
        AK_CUDA(cudaEventRecord(c->ev_join, c->side));
        AK_CUDA(cudaStreamWaitEvent(c->stream, c->ev_join, 0));
    }
    // bulk (scheduled while the boundary kernels drain; it waits for them)
    mark(c);
    const unsigned grid = stream_collide_grid<S>(make_int4(0, 0, 0, 0), c->nx, c->ny, c->nz);
    AK_CUDA(launch_chained(CHAIN_UNIFORM, k_stream_collide<S, false>, dim3(grid), dim3(128), c->stream, (const S *)src,
                           dst_of<S>(c), (const uint8_t *)c->flags, c->G, c->shift_host, (T)c->omega_s,
                           (T)c->omega_b, sgs_of<S>(c), make_int4(0, 0, 0, 0), make_int4(0, 0, 0, 0),
                           make_int4(0, 0, 0, 0), (long long *)nullptr));
    ++c->launches;
    mark(c);
    c->cur = 1 - c->cur;
    c->steps += 1;
    return AK_OK;
}

// One step replayed from the captured graph of its (copy parity, sample) slot.
template <typename S>
int step_graphed(ak_case *c, bool sample) {
    const long long nlinks = c->nkeys * c->nz * 3;
    if (sample && nlinks) AK_TRY(ensure_partials(c, blocks_for(nlinks, 256) * 5 * c->n_elements));
    if (!c->side) {
        if (cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess)
            return fail(AK_ERR_CUDA, "stream or event creation failed");
    }
    // the exterior step samples its loads every step and flips its band
    // buffers with the population copies: its slot is the two parities
    const int slot = c->farfield == AK_FARFIELD_EXTERIOR ? (c->cur | (c->ext_cur << 1)) : (c->cur | (sample ? 2 : 0));
    if (c->step_graph[slot] && c->graph_partials[slot] != c->partials) {
        cudaGraphExecDestroy(c->step_graph[slot]);
        c->step_graph[slot] = nullptr;
    }
    if (!c->step_graph[slot]) {
        const int cur = c->cur, ext_cur = c->ext_cur;
        const long long steps = c->steps, launches = c->launches;
        AK_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        const int r = one_step<S>(c, sample, nullptr, 0, true);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        const long long per = c->launches - launches;
        c->cur = cur;
        c->ext_cur = ext_cur;
        c->steps = steps;
        c->launches = launches;
        if (r != AK_OK || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            return r != AK_OK ? r : fail(AK_ERR_CUDA, std::string("step capture failed: ") + cudaGetErrorString(e));
        }
        const cudaError_t ei = cudaGraphInstantiate(&c->step_graph[slot], g, 0);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) {
            c->step_graph[slot] = nullptr;
            return fail(AK_ERR_CUDA, std::string("step graph instantiation failed: ") + cudaGetErrorString(ei));
        }
        c->graph_partials[slot] = c->partials;
        c->graph_launches[slot] = per;
    }
    AK_CUDA(cudaGraphLaunch(c->step_graph[slot], c->stream));
    c->cur = 1 - c->cur;
    if (c->farfield == AK_FARFIELD_EXTERIOR) c->ext_cur = 1 - c->ext_cur;
    c->steps += 1;
    c->launches += c->graph_launches[slot];
    return AK_OK;
}

// One step of the exterior farfield (exterior.py:173-200 around solver.py:
// 262-271): the ring predictor from the current band state, the walls with
// their loads and wall mass (every step: the wall mass accumulates), the
// streamed band macros, the rebuilt and collided ring, the fused bulk
// stream-collide, and the step's source and wall-mass sums.
template <typename S>
int exterior_step(ak_case *c, double *fixed_partials, long long fixed_capacity, bool branch) {
    using T = typename Store<S>::T;
    if (!c->prepared) return fail(AK_ERR_INVALID, "the exterior case needs an initial state first");
    // branch (captured graphs): the walls on the side stream beside the
    // predictor, joined before the band pull (which may read a solid cell of
    // the third layer) -- the step's clock lives on the device (ext_out[11])
    S *src = src_of<S>(c), *dst = dst_of<S>(c);
    const ExtGeom &E = c->ext;
    double *band = c->ext_band[c->ext_cur], *next = c->ext_band[1 - c->ext_cur];
    const long long nr = (long long)E.nring * E.nz;
    // 64-thread blocks over the ~2 (nx + ny) nz ring cells: the FP64 ring
    // arithmetic spreads over every SM
    const unsigned rb = (unsigned)blocks_for(nr, EXT_THREADS);
    const double *clock = c->ext_out + 11;
    cudaStream_t ws = c->stream;
    if (branch) {
        AK_CUDA(cudaEventRecord(c->ev_fork, c->stream));
        AK_CUDA(cudaStreamWaitEvent(c->side, c->ev_fork, 0));
        ws = c->side;
    }
    mark(c);
    double *moment_error = c->ext_out + 10;
    k_ext_stage<<<rb, EXT_THREADS, 0, c->stream>>>(E, band, nullptr, c->ext_stage[0], 1, clock, c->ext_inc0,
                                                   moment_error);
    k_ext_stage<<<rb, EXT_THREADS, 0, c->stream>>>(E, band, c->ext_stage[0], c->ext_stage[1], 2, clock,
                                                   c->ext_inc0, moment_error);
    k_ext_stage<<<rb, EXT_THREADS, 0, c->stream>>>(E, band, c->ext_stage[1], c->ext_stage[2], 3, clock,
                                                   c->ext_inc0, moment_error);
    AK_CUDA(cudaGetLastError());
    c->launches += 3;
    mark(c);
    const long long nlinks = c->nkeys * c->nz * 3;
    if (nlinks) {
        const long long nb = c->wall_blocks;
        double *partials = c->partials;
        if (fixed_partials) {
            if (nb * 5 * c->n_elements > fixed_capacity)
                return fail(AK_ERR_INVALID, "wall links need more partial sums than the static scratch holds");
            partials = fixed_partials;
        }
        k_walls<S><<<(unsigned)nb, 256, 0, ws>>>(src, c->G, c->keys, c->wall_q, c->nkeys, 1, c->n_elements, c->ox,
                                                 c->oy, partials);
        k_sum_partials<<<5 * c->n_elements, 32, 0, ws>>>(partials, (int)nb, 5 * c->n_elements, c->reduced);
        AK_CUDA(cudaGetLastError());
        c->launches += 2;
    } else {
        AK_CUDA(cudaMemsetAsync(c->reduced, 0, sizeof(double) * 5 * c->n_elements, ws));
    }
    if (branch) {
        AK_CUDA(cudaEventRecord(c->ev_join, c->side));
        AK_CUDA(cudaStreamWaitEvent(c->stream, c->ev_join, 0));
    }
    mark(c);
    k_ext_band_pull<S><<<(unsigned)blocks_for((long long)E.nband * E.nz, 128), 128, 0, c->stream>>>(src, c->G, E,
                                                                                                    next);
    k_ext_ring<S><<<rb, EXT_THREADS, 0, c->stream>>>(src, dst, c->G, E, next, c->ext_stage[2], c->shift_host,
                                                     (T)c->omega_s, (T)c->omega_b, c->omega_s, c->ext_partials,
                                                     moment_error);
    AK_CUDA(cudaGetLastError());
    c->launches += 2;
    mark(c);
    const unsigned grid = stream_collide_grid<S>(make_int4(0, 0, 0, 0), c->nx, c->ny, c->nz);
    k_stream_collide<S><<<grid, 128, 0, c->stream>>>(src, dst, c->flags, c->G, c->shift_host, (T)c->omega_s,
                                                     (T)c->omega_b, Sgs<T>{});
    AK_CUDA(cudaGetLastError());
    mark(c);
    k_ext_final<<<1, REDUCE_THREADS, 0, c->stream>>>(c->ext_partials, rb, c->reduced, c->n_elements, c->ext_out);
    AK_CUDA(cudaGetLastError());
    c->launches += 2;
    c->cur = 1 - c->cur;
    c->ext_cur = 1 - c->ext_cur;
    c->steps += 1;
    return AK_OK;
}

// The initial exterior state: the ring at the freestream equilibrium, the
// band state and the glancing rows' invariant of these pre-collision
// populations, then their collision into the stored (post-collision) form.
template <typename S>
int exterior_prepare(ak_case *c) {
    using T = typename Store<S>::T;
    S *pdf = src_of<S>(c);
    const ExtGeom &E = c->ext;
    const long long nr = (long long)E.nring * E.nz;
    k_ext_fill_ring<S><<<(unsigned)blocks_for(nr, 128), 128, 0, c->stream>>>(pdf, c->G, E);
    k_ext_band_direct<S><<<(unsigned)blocks_for((long long)E.nband * E.nz, 128), 128, 0, c->stream>>>(
        pdf, c->G, E, c->ext_band[0], c->ext_inc0);
    k_collide<S><<<(unsigned)blocks_for((long long)c->nx * c->ny * c->nz, 128), 128, 0, c->stream>>>(
        pdf, c->flags, c->G, c->shift_host, (T)c->omega_s, (T)c->omega_b);
    k_ext_collide_ring<S><<<(unsigned)blocks_for(nr, 128), 128, 0, c->stream>>>(pdf, c->G, E, c->shift_host,
                                                                                (T)c->omega_s, (T)c->omega_b);
    AK_CUDA(cudaGetLastError());
    AK_CUDA(cudaMemsetAsync(c->ext_out, 0, 12 * sizeof(double), c->stream));
    c->ext_cur = 0;
    c->prepared = true;
    return AK_OK;
}

// the two layers inside the ring must be fluid (the plan keeps two fluid
// cells between the body and the physical edge; the ring itself is the ghost
// layer, flagged outer and free of solids by build_geometry); the buffers of
// the ring work
int build_exterior(ak_case *c, const std::vector<uint8_t> &hflags) {
    c->ext = make_ext_geom(c->nx, c->ny, c->nz, c->speed);
    const ExtGeom &E = c->ext;
    if (E.NX < 6 || E.NY < 6) return fail(AK_ERR_INVALID, "the exterior farfield needs at least 4 cells in x and y");
    for (int y = 0; y < E.NY; ++y)
        for (int x = 0; x < E.NX; ++x) {
            const int layer = std::min(std::min(x, y), std::min(E.NX - 1 - x, E.NY - 1 - y));
            if (layer >= 1 && layer <= 2 && hflags[(size_t)y * c->G.nxp + x] != FLAG_FLUID)
                return fail(AK_ERR_INVALID, "the two layers inside the exterior ring must be fluid");
        }
    const long long nr = (long long)E.nring * E.nz, nb = (long long)E.nband * E.nz;
    for (int k = 0; k < 2; ++k) AK_TRY(dalloc(c, &c->ext_band[k], 4 * nb));
    for (int k = 0; k < 3; ++k) AK_TRY(dalloc(c, &c->ext_stage[k], 4 * nr));
    AK_TRY(dalloc(c, &c->ext_inc0, 2LL * E.nz * E.NX));
    c->ext_blocks = blocks_for(nr, EXT_THREADS);
    AK_TRY(dalloc(c, &c->ext_partials, 4 * c->ext_blocks));
    AK_TRY(dalloc(c, &c->ext_out, 12));
    AK_CUDA(cudaMemsetAsync(c->ext_out, 0, 12 * sizeof(double), c->stream));
    // the walls reduce their loads every step: size the partials once
    c->wall_blocks = blocks_for(c->nkeys * c->nz * 3, 256);
    if (c->wall_blocks) AK_TRY(ensure_partials(c, c->wall_blocks * 5 * c->n_elements));
    return AK_OK;
}

int check_case(const ak_case *c) {
    if (!c) return fail(AK_ERR_INVALID, "null case");
    return AK_OK;
}

}  // namespace

extern "C" {

const char *ak_last_error(void) { return g_error.c_str(); }

const char *ak_version(void) {
#ifdef AK_CHECKED
    return "aerokinetic_gb300 1.0 sm_103a checked";
#else
    return "aerokinetic_gb300 1.0 sm_103a";
#endif
}

int ak_fma_peak(int32_t precision, double *tflops) {
    if (precision < 0 || precision > 2 || !tflops)
        return fail(AK_ERR_INVALID, "precision 0 (FP64), 1 (FP32) or 2 (packed FP32x2) and an output are required");
    int dev = 0, sms = 0;
    AK_CUDA(cudaGetDevice(&dev));
    AK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int threads = 256, blocks = 8 * sms;
    // about 30 ms per launch on GB300 for either pipe
    const int iters = precision == 0 ? 8192 : 262144;
    cudaStream_t st = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    void *out = nullptr;
    AK_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    int r = AK_OK;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess ||
        cudaMalloc(&out, (size_t)blocks * threads * 8) != cudaSuccess)
        r = fail(AK_ERR_CUDA, "peak measurement set-up failed");
    double best = 0.0;
    for (int rep = 0; rep < 4 && r == AK_OK; ++rep) {
        cudaEventRecord(a, st);
        if (precision == 0)
            k_fma_peak<double><<<blocks, threads, 0, st>>>((double *)out, iters, 0.999999, 1e-6);
        else if (precision == 1)
            k_fma_peak<float><<<blocks, threads, 0, st>>>((float *)out, iters, 0.999999f, 1e-6f);
        else
            k_fma2_peak<<<blocks, threads, 0, st>>>((float *)out, iters, 0.999999f, 1e-6f);
        cudaEventRecord(b, st);
        if (cudaEventSynchronize(b) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
            r = fail(AK_ERR_CUDA, "peak measurement kernel failed");
            break;
        }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, a, b);
        const double flops = (precision == 2 ? 4.0 : 2.0) * 8.0 * (double)iters * blocks * threads;
        if (rep > 0) best = std::max(best, flops / (ms * 1e-3) / 1e12);  // the first launch warms up
    }
    if (out) cudaFree(out);
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    cudaStreamDestroy(st);
    if (r != AK_OK) return r;
    *tflops = best;
    return AK_OK;
}

int ak_collision_flops(int32_t storage, double *counts) {
    if (storage < AK_STORAGE_F64 || storage > AK_STORAGE_F16 || !counts)
        return fail(AK_ERR_INVALID, "storage f64, f32 or f16 and an output are required");
    // any non-degenerate cell: the operation count does not depend on the values
    Counted g[Q];
    for (int q = 0; q < Q; ++q) g[q] = Counted(1e-3 * ((q * 7) % 11 - 5) * weight(q));
    Counted::reset();
    // the collision form each storage type uses (collide_stored)
    if (storage == AK_STORAGE_F32)
        collide<Counted>(g, Counted(1.9), Counted(1.0));
    else
        collide_full<Counted>(g, Counted(1.0 - 1.9), Counted(1.0));
    counts[0] = (double)Counted::adds;
    counts[1] = (double)Counted::muls;
    counts[2] = (double)Counted::divs;
    counts[3] = (double)(Counted::adds + Counted::muls + Counted::divs);
    return AK_OK;
}

#ifdef AK_CHECKED
unsigned long long ak_debug_status(void) {
    unsigned long long v = 0, zero = 0;
    cudaDeviceSynchronize();
    cudaMemcpyFromSymbol(&v, ak_debug_word, sizeof v);
    cudaMemcpyToSymbol(ak_debug_word, &zero, sizeof zero);
    return v;
}
#endif

}  // extern "C"

namespace {
// Builds a lattice from a validated description.  farfield -1 = no outer
// boundary (the refined fine block), periodic_xy wraps x and y.
int create_lattice(const ak_case_desc *desc, int farfield, bool periodic_xy, ak_case **out) {
    *out = nullptr;
    ak_case *c = new ak_case();
    c->nx = desc->nx;
    c->ny = desc->ny;
    c->nz = desc->nz;
    c->res_region[1] = desc->nx;
    c->res_region[3] = desc->ny;
    c->origin_x = desc->origin_x;
    c->origin_y = desc->origin_y;
    c->dx = desc->dx;
    c->ox = desc->origin_x / desc->dx;
    c->oy = desc->origin_y / desc->dx;
    c->omega_s = desc->omega_shear;
    c->omega_b = desc->omega_bulk;
    c->smagorinsky = desc->smagorinsky;
    c->speed = desc->speed;
    c->farfield = farfield;
    c->periodic_xy = periodic_xy;
    c->storage = desc->storage;
    c->n_elements = desc->n_elements;
    int total = 0;
    for (int e = 0; e < desc->n_elements; ++e) {
        if (desc->element_sizes[e] < 3) {
            delete c;
            return fail(AK_ERR_INVALID, "a polygon needs at least three vertices");
        }
        c->poly_start.push_back(total);
        c->poly_count.push_back(desc->element_sizes[e]);
        total += desc->element_sizes[e];
    }
    if (total) c->poly_xy.assign(desc->polygon_xy, desc->polygon_xy + 2 * (size_t)total);
    for (double v : c->poly_xy)
        if (!std::isfinite(v)) {
            delete c;
            return fail(AK_ERR_INVALID, "polygon vertices must be finite");
        }
    c->esize = (c->storage == AK_STORAGE_F64 || c->storage == AK_STORAGE_DF64) ? 8 : (c->storage == AK_STORAGE_F32 ? 4 : 2);
    Grid &G = c->G;
    G.nx = c->nx;
    G.ny = c->ny;
    G.nz = c->nz;
    G.nxp = c->nx + 2;
    G.nyp = c->ny + 2;
    G.sx = (G.nxp + 31) / 32 * 32;
    G.plane = (long long)G.nyp * G.sx;
    G.qs = (long long)G.nz * G.plane;
    std::vector<float> shift(Q);
    for (int q = 0; q < Q; ++q) {
        // zero-centred equilibrium of the freestream (1, (U, 0, 0)), the FP16 shift
        const double u[3] = {c->speed, 0.0, 0.0};
        const int e[3] = {cx(q), cy(q), cz(q)};
        double p = 1.0;
        for (int a = 0; a < 3; ++a)
            p *= e[a] == 0 ? 2.0 / 3.0 - u[a] * u[a] : 0.5 * (1.0 / 3.0 + u[a] * u[a] + e[a] * u[a]);
        shift[q] = c->storage == AK_STORAGE_F16 ? (float)(p - weight(q)) : 0.0f;
        c->shift_host.v[q] = shift[q];
    }
    int r = AK_OK;
    if (cudaGetDevice(&c->device) != cudaSuccess) r = fail(AK_ERR_CUDA, "no current CUDA device");
    if (r == AK_OK && cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        r = fail(AK_ERR_CUDA, "stream creation failed (no CUDA device?)");
    }
    if (r == AK_OK) r = upload(c, &c->d_shift, shift);
    G.shift = c->d_shift;
    std::vector<uint8_t> hflags;
    if (r == AK_OK && c->farfield == AK_FARFIELD_CHARACTERISTIC) build_farfield_objects(c);
    if (r == AK_OK) r = build_geometry(c, hflags);
    if (r == AK_OK && c->farfield == AK_FARFIELD_EXTERIOR) r = build_exterior(c, hflags);
    else if (r == AK_OK && c->farfield >= 0) r = build_outer(c, hflags);
    if (r == AK_OK) r = dalloc(c, &c->reduced, 64);
    if (r == AK_OK) r = with_storage(c, [&](auto *tag) { return allocate_populations<std::remove_pointer_t<decltype(tag)>>(c); });
    if (r == AK_OK && cudaStreamSynchronize(c->stream) != cudaSuccess) r = fail(AK_ERR_CUDA, "case set-up failed");
    if (r != AK_OK) {
        std::string keep = g_error;
        release(c);
        delete c;
        g_error = keep;
        return r;
    }
    *out = c;
    return AK_OK;
}

int validate_desc(const ak_case_desc *desc, bool need_elements) {
    if (desc->nx < 4 || desc->ny < 4 || desc->nz < 1) return fail(AK_ERR_INVALID, "lattice needs nx, ny >= 4 and nz >= 1");
    if ((long long)desc->nx + 2 > 32767 || (long long)desc->ny + 2 > 65535 || desc->nz > 65535)
        return fail(AK_ERR_INVALID, "lattice extent too large for one case");
    if (!(desc->dx > 0) || !std::isfinite(desc->dx)) return fail(AK_ERR_INVALID, "dx must be positive");
    if (!(desc->omega_shear > 0 && desc->omega_shear < 2) || !(desc->omega_bulk > 0 && desc->omega_bulk < 2))
        return fail(AK_ERR_INVALID, "relaxation rates must lie in (0, 2)");
    if (!std::isfinite(desc->speed) || std::fabs(desc->speed) >= 1.0 / std::sqrt(3.0))
        return fail(AK_ERR_INVALID, "freestream speed must be subsonic");
    if (desc->farfield != AK_FARFIELD_LEGACY && desc->farfield != AK_FARFIELD_CHARACTERISTIC &&
        desc->farfield != AK_FARFIELD_EXTERIOR)
        return fail(AK_ERR_INVALID, "unknown farfield");
    if (desc->storage < AK_STORAGE_F64 || desc->storage > AK_STORAGE_DF64) return fail(AK_ERR_INVALID, "unknown storage");
    if (!(desc->smagorinsky >= 0.0 && desc->smagorinsky < 0.3))
        return fail(AK_ERR_INVALID, "the Smagorinsky constant must lie in [0, 0.3)");
    if (desc->smagorinsky > 0.0 && desc->farfield == AK_FARFIELD_EXTERIOR)
        return fail(AK_ERR_INVALID, "Exterior FD currently supports molecular viscosity with sgs=none only");
    if ((need_elements && desc->n_elements < 1) || desc->n_elements > MAX_ELEMENTS ||
        (desc->n_elements && (!desc->element_sizes || !desc->polygon_xy)))
        return fail(AK_ERR_INVALID, "between 1 and 8 polygons are required");
    return AK_OK;
}
}  // namespace

extern "C" {

int ak_case_create(const ak_case_desc *desc, ak_case **out) {
    g_error.clear();
    if (!desc || !out) return fail(AK_ERR_INVALID, "null argument");
    *out = nullptr;
    AK_TRY(validate_desc(desc, true));
    return create_lattice(desc, desc->farfield, false, out);
}

int ak_case_destroy(ak_case *c) {
    if (!c) return AK_OK;
    cudaStreamSynchronize(c->stream);
    release(c);
    delete c;
    return AK_OK;
}

int ak_case_get_info(const ak_case *c, ak_case_info *info) {
    AK_TRY(check_case(c));
    if (!info) return fail(AK_ERR_INVALID, "null info");
    info->cells = (int64_t)c->nx * c->ny * c->nz;
    info->fluid_cells = c->fluid_cells;
    info->wall_keys = c->nkeys;
    info->wall_links = c->nkeys * c->nz * 3;
    info->outer_links = c->nouter;
    info->fallback_links = c->fallback;
    info->device_bytes = (int64_t)c->device_bytes;
    info->row_pitch = c->G.sx;
    info->storage = c->storage;
    return AK_OK;
}

int ak_init_perturbed(ak_case *c, double amp, double phase_y, double phase_z, double lead_x, double lead_y,
                      double span) {
    AK_TRY(check_case(c));
    if (!(span > 0)) return fail(AK_ERR_INVALID, "span must be positive");
    const double ky = 2 * M_PI / (c->ny * c->dx);
    const double kz = 2 * M_PI / span;
    const long long n = (long long)c->nx * c->ny * c->nz;
    AK_TRY(with_storage(c, [&](auto *tag) {
        using S = std::remove_pointer_t<decltype(tag)>;
        k_init_perturbed<S><<<(unsigned)blocks_for(n, 256), 256, 0, c->stream>>>(
            src_of<S>(c), c->G, c->flags, c->speed, amp, phase_y, phase_z, lead_x, lead_y, c->origin_x, c->origin_y,
            c->dx, ky, kz);
        AK_CUDA(cudaGetLastError());
        if (c->farfield == AK_FARFIELD_EXTERIOR) return exterior_prepare<S>(c);
        return AK_OK;
    }));
    AK_CUDA(cudaStreamSynchronize(c->stream));
    c->prepared = c->farfield == AK_FARFIELD_EXTERIOR;
    c->steps = 0;
    ++c->pdf_writes;
    return AK_OK;
}

int ak_init_fields(ak_case *c, const double *rho, const double *u) {
    AK_TRY(check_case(c));
    if (!rho || !u) return fail(AK_ERR_INVALID, "null field");
    const long long n = (long long)c->nx * c->ny * c->nz;
    AK_TRY(ensure_staging(c, (size_t)n * 4));
    AK_CUDA(cudaMemcpyAsync(c->staging, rho, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    AK_CUDA(cudaMemcpyAsync(c->staging + n, u, 3 * n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    AK_TRY(with_storage(c, [&](auto *tag) {
        using S = std::remove_pointer_t<decltype(tag)>;
        k_init_fields<S><<<(unsigned)blocks_for(n, 256), 256, 0, c->stream>>>(src_of<S>(c), c->G, c->staging,
                                                                               c->staging + n);
        AK_CUDA(cudaGetLastError());
        if (c->farfield == AK_FARFIELD_EXTERIOR) return exterior_prepare<S>(c);
        return AK_OK;
    }));
    AK_CUDA(cudaStreamSynchronize(c->stream));
    c->prepared = c->farfield == AK_FARFIELD_EXTERIOR;
    c->steps = 0;
    ++c->pdf_writes;
    return AK_OK;
}

int ak_step(ak_case *c, int32_t nsteps, double *loads) {
    AK_TRY(check_case(c));
    if (nsteps < 1) return fail(AK_ERR_INVALID, "nsteps must be >= 1");
    for (int s = 0; s < nsteps; ++s) {
        const bool sample = loads != nullptr && s == nsteps - 1;
        AK_TRY(with_storage(c, [&](auto *tag) {
            using S = std::remove_pointer_t<decltype(tag)>;
            // the first step prepares the boundaries eagerly; timed steps
            // stay eager
            if (c->prepared && !c->timing) return step_graphed<S>(c, sample);
            return one_step<S>(c, sample);
        }));
    }
    if (loads) {
        AK_CUDA(cudaMemcpyAsync(loads, c->reduced, sizeof(double) * 5 * c->n_elements, cudaMemcpyDeviceToHost,
                                c->stream));
        AK_CUDA(cudaStreamSynchronize(c->stream));
    }
    return AK_OK;
}

}  // extern "C"

// ---- allocation-free loads
// Some callers cannot allocate device memory once they run: a host
// application whose memory pool has already reserved the GPU's free memory
// (a cudaMalloc would fail or fragment its pool), a control loop on a fixed
// device budget that cannot afford the implicit synchronisation of an
// allocation, or a plugin host that forbids driver allocations after
// start-up.  ak_step's loads path allocates its per-block partial sums on
// the first sampled step; ak_step_loads_static keeps them in this file-scope
// array instead: 131072 doubles (1 MiB) that every GPU loading the library
// holds until the process exits.  It steps eagerly (one launch per kernel,
// no graph replay), so each step costs the launch latencies ak_step's
// replayed graphs hide.
namespace {
constexpr long long STATIC_LOADS_DOUBLES = 131072;
constexpr int STATIC_MAX_DEVICES = 64;
std::mutex g_static_mutex;
double *g_static_address[STATIC_MAX_DEVICES] = {nullptr};
}  // namespace
static __device__ __align__(256) double g_static_loads[STATIC_LOADS_DOUBLES];

namespace {
// Device address of the scratch array for the current device, looked up once
// per device (the host-side symbol is only a stand-in, never a device address).
int static_loads_scratch(double **out) {
    int dev = 0;
    AK_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= STATIC_MAX_DEVICES) return fail(AK_ERR_INVALID, "device index out of range");
    std::lock_guard<std::mutex> lock(g_static_mutex);
    if (!g_static_address[dev]) {
        void *ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_static_loads);
        if (e != cudaSuccess)
            return fail(AK_ERR_CUDA, std::string("cudaGetSymbolAddress of the static scratch failed: ") +
                                         cudaGetErrorString(e));
        g_static_address[dev] = (double *)ptr;
    }
    *out = g_static_address[dev];
    return AK_OK;
}
}  // namespace

extern "C" {

int ak_step_loads_static(ak_case *c, int32_t nsteps, double *loads) {
    AK_TRY(check_case(c));
    if (nsteps < 1 || !loads) return fail(AK_ERR_INVALID, "nsteps >= 1 and a loads array are required");
    int dev = 0;
    AK_CUDA(cudaGetDevice(&dev));
    if (dev != c->device)
        return fail(AK_ERR_INVALID, "make the case's device current before ak_step_loads_static");
    // every check before the first launch: a rejected call leaves the case,
    // its boundary history and its step count as they were
    if (c->farfield == AK_FARFIELD_EXTERIOR && !c->prepared)
        return fail(AK_ERR_INVALID, "the exterior case needs an initial state first");
    const long long blocks =
        c->farfield == AK_FARFIELD_EXTERIOR ? c->wall_blocks : blocks_for(c->nkeys * c->nz * 3, 256);
    const long long needed = blocks * 5 * c->n_elements;
    if (needed > STATIC_LOADS_DOUBLES)
        return fail(AK_ERR_INVALID, "wall links need " + std::to_string(needed) +
                                        " partial sums; the static scratch holds " +
                                        std::to_string(STATIC_LOADS_DOUBLES));
    double *scratch = nullptr;
    AK_TRY(static_loads_scratch(&scratch));
    for (int s = 0; s < nsteps; ++s) {
        const bool sample = s == nsteps - 1;
        AK_TRY(with_storage(c, [&](auto *tag) {
            return one_step<std::remove_pointer_t<decltype(tag)>>(c, sample, scratch, STATIC_LOADS_DOUBLES);
        }));
    }
    AK_CUDA(cudaMemcpyAsync(loads, c->reduced, sizeof(double) * 5 * c->n_elements, cudaMemcpyDeviceToHost,
                            c->stream));
    AK_CUDA(cudaStreamSynchronize(c->stream));
    return AK_OK;
}

int64_t ak_steps_done(const ak_case *c) { return c ? c->steps : -1; }

int64_t ak_kernel_launches(const ak_case *c) { return c ? c->launches : -1; }

void *ak_case_stream(const ak_case *c) { return c ? (void *)c->stream : nullptr; }

int ak_step_timed(ak_case *c, int32_t nsteps, double *ms) {
    AK_TRY(check_case(c));
    if (nsteps < 1 || !ms) return fail(AK_ERR_INVALID, "nsteps >= 1 and an output array are required");
    // events per step: outer boundary | walls | stream-collide; the exterior
    // step has a fourth interval (the ring rebuild, part of its outer boundary)
    const int marks = c->farfield == AK_FARFIELD_EXTERIOR ? 5 : 4;
    std::vector<cudaEvent_t> events;
    events.reserve((size_t)marks * nsteps);
    c->timing = &events;
    int r = AK_OK;
    for (int s = 0; s < nsteps && r == AK_OK; ++s)
        r = with_storage(c, [&](auto *tag) { return one_step<std::remove_pointer_t<decltype(tag)>>(c, false); });
    c->timing = nullptr;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    for (int k = 0; k < 4; ++k) ms[k] = 0.0;
    if (r == AK_OK && e == cudaSuccess && events.size() == (size_t)marks * nsteps) {
        float t = 0.0f;
        cudaEventElapsedTime(&t, events.front(), events.back());
        ms[0] = t;
        for (int s = 0; s < nsteps; ++s) {
            cudaEvent_t *ev = events.data() + marks * s;
            cudaEventElapsedTime(&t, ev[0], ev[1]);  // outer boundary (exterior: the predictor)
            ms[3] += t;
            cudaEventElapsedTime(&t, ev[1], ev[2]);  // walls
            ms[2] += t;
            if (marks == 5) {
                cudaEventElapsedTime(&t, ev[2], ev[3]);  // exterior: band state and ring rebuild
                ms[3] += t;
            }
            cudaEventElapsedTime(&t, ev[marks - 2], ev[marks - 1]);  // stream-collide
            ms[1] += t;
        }
    }
    for (cudaEvent_t ev : events) cudaEventDestroy(ev);
    if (r != AK_OK) return r;
    AK_CUDA(e);
    return AK_OK;
}

int ak_diagnostics(ak_case *c, double *diag) {
    AK_TRY(check_case(c));
    if (!diag) return fail(AK_ERR_INVALID, "null output");
    const int nb = 152 * 4;
    const int ring_rows = c->farfield == AK_FARFIELD_EXTERIOR ? 64 : 0;
    AK_TRY(ensure_partials(c, (long long)(nb + ring_rows) * 6));
    AK_TRY(with_storage(c, [&](auto *tag) {
        using S = std::remove_pointer_t<decltype(tag)>;
        k_diagnostics<S><<<nb, 256, 0, c->stream>>>(src_of<S>(c), c->G, c->flags, c->partials);
        if (ring_rows)
            k_ext_ring_diagnostics<S><<<ring_rows, 256, 0, c->stream>>>(src_of<S>(c), c->G, c->ext,
                                                                         c->partials + (long long)nb * 6);
        AK_CUDA(cudaGetLastError());
        return AK_OK;
    }));
    k_diagnostics_final<<<1, REDUCE_THREADS, 0, c->stream>>>(c->partials, nb + ring_rows, c->reduced);
    AK_CUDA(cudaGetLastError());
    double r[6];
    AK_CUDA(cudaMemcpyAsync(r, c->reduced, sizeof r, cudaMemcpyDeviceToHost, c->stream));
    AK_CUDA(cudaStreamSynchronize(c->stream));
    diag[0] = std::sqrt(3.0) * std::sqrt(r[0]);
    diag[1] = r[5] > 0 ? r[3] / r[5] : NAN;
    diag[2] = r[1];
    diag[3] = -r[2];
    diag[4] = (r[4] == 0 && r[5] > 0) ? 1.0 : 0.0;
    if (diag[4] != 1.0) return fail(AK_ERR_NONFINITE, "Non-finite fluid state; the run is invalid");
    if (diag[0] > 0.3 || diag[2] > 0.1 || diag[3] <= 0) {
        char buf[160];
        std::snprintf(buf, sizeof buf, "Low-Mach validity check failed: local Ma=%.3g, |rho-1|max=%.3g", diag[0],
                      diag[2]);
        return fail(AK_ERR_GUARD, buf);
    }
    return AK_OK;
}

int ak_macros(ak_case *c, double *rho, double *u) {
    AK_TRY(check_case(c));
    if (!rho || !u) return fail(AK_ERR_INVALID, "null output");
    const long long n = (long long)c->nx * c->ny * c->nz;
    AK_TRY(ensure_staging(c, (size_t)n * 4));
    AK_TRY(with_storage(c, [&](auto *tag) {
        using S = std::remove_pointer_t<decltype(tag)>;
        k_macros<S><<<(unsigned)blocks_for(n, 256), 256, 0, c->stream>>>(src_of<S>(c), c->G, c->staging,
                                                                          c->staging + n);
        AK_CUDA(cudaGetLastError());
        return AK_OK;
    }));
    AK_CUDA(cudaMemcpyAsync(rho, c->staging, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    AK_CUDA(cudaMemcpyAsync(u, c->staging + n, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    AK_CUDA(cudaStreamSynchronize(c->stream));
    return AK_OK;
}

int ak_get_pdf(ak_case *c, double *pdf) {
    AK_TRY(check_case(c));
    if (!pdf) return fail(AK_ERR_INVALID, "null output");
    const long long n = (long long)c->nx * c->ny * c->nz;
    AK_TRY(ensure_staging(c, (size_t)n * Q));
    AK_TRY(with_storage(c, [&](auto *tag) {
        using S = std::remove_pointer_t<decltype(tag)>;
        k_export<S><<<(unsigned)blocks_for(n, 256), 256, 0, c->stream>>>(src_of<S>(c), c->G, c->staging);
        AK_CUDA(cudaGetLastError());
        return AK_OK;
    }));
    AK_CUDA(cudaMemcpyAsync(pdf, c->staging, n * Q * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    AK_CUDA(cudaStreamSynchronize(c->stream));
    return AK_OK;
}

int ak_set_pdf(ak_case *c, const double *pdf) {
    AK_TRY(check_case(c));
    if (!pdf) return fail(AK_ERR_INVALID, "null input");
    const long long n = (long long)c->nx * c->ny * c->nz;
    AK_TRY(ensure_staging(c, (size_t)n * Q));
    AK_CUDA(cudaMemcpyAsync(c->staging, pdf, n * Q * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    AK_TRY(with_storage(c, [&](auto *tag) {
        using S = std::remove_pointer_t<decltype(tag)>;
        k_import<S><<<(unsigned)blocks_for(n, 256), 256, 0, c->stream>>>(src_of<S>(c), c->G, c->staging);
        AK_CUDA(cudaGetLastError());
        return AK_OK;
    }));
    ++c->pdf_writes;
    AK_CUDA(cudaStreamSynchronize(c->stream));
    return AK_OK;
}

// ---- outer-boundary history for checkpoints
namespace {
// exterior state: ring populations (ring cell, z, 27), the current band state,
// the glancing rows' initial invariant and the running sums
long long exterior_values(const ak_case *c) {
    const ExtGeom &E = c->ext;
    return (long long)E.nring * E.nz * Q + 4LL * E.nband * E.nz + 2LL * E.NX * E.nz + 10;
}
int exterior_state(ak_case *c, double *v, bool write) {
    const ExtGeom &E = c->ext;
    const long long nr = (long long)E.nring * E.nz, nb = 4LL * E.nband * E.nz, ni = 2LL * E.NX * E.nz;
    AK_TRY(ensure_staging(c, (size_t)(nr * Q)));
    if (write) {
        for (long long k = 0; k < exterior_values(c); ++k)
            if (!std::isfinite(v[k])) return fail(AK_ERR_INVALID, "exterior state is not finite");
        AK_CUDA(cudaMemcpyAsync(c->staging, v, nr * Q * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    }
    AK_TRY(with_storage(c, [&](auto *tag) {
        using S = std::remove_pointer_t<decltype(tag)>;
        if (write)
            k_ext_ring_import<S><<<(unsigned)blocks_for(nr, 128), 128, 0, c->stream>>>(src_of<S>(c), c->G, E,
                                                                                      c->staging);
        else
            k_ext_ring_export<S><<<(unsigned)blocks_for(nr, 128), 128, 0, c->stream>>>(src_of<S>(c), c->G, E,
                                                                                      c->staging);
        AK_CUDA(cudaGetLastError());
        return AK_OK;
    }));
    const cudaMemcpyKind kind = write ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
    double *band = c->ext_band[c->ext_cur];
    if (write) {
        AK_CUDA(cudaMemcpyAsync(band, v + nr * Q, nb * sizeof(double), kind, c->stream));
        AK_CUDA(cudaMemcpyAsync(c->ext_inc0, v + nr * Q + nb, ni * sizeof(double), kind, c->stream));
        AK_CUDA(cudaMemcpyAsync(c->ext_out, v + nr * Q + nb + ni, 10 * sizeof(double), kind, c->stream));
    } else {
        AK_CUDA(cudaMemcpyAsync(v, c->staging, nr * Q * sizeof(double), kind, c->stream));
        AK_CUDA(cudaMemcpyAsync(v + nr * Q, band, nb * sizeof(double), kind, c->stream));
        AK_CUDA(cudaMemcpyAsync(v + nr * Q + nb, c->ext_inc0, ni * sizeof(double), kind, c->stream));
        AK_CUDA(cudaMemcpyAsync(v + nr * Q + nb + ni, c->ext_out, 10 * sizeof(double), kind, c->stream));
    }
    AK_CUDA(cudaStreamSynchronize(c->stream));
    return AK_OK;
}

long long boundary_values(const ak_case *c) {
    if (c->farfield == AK_FARFIELD_CHARACTERISTIC) return 1 + 3 * c->nouter + 2LL * c->nx * c->nz;
    if (c->farfield == AK_FARFIELD_LEGACY) return 1 + 2 * c->n_out;
    if (c->farfield == AK_FARFIELD_EXTERIOR) return 1 + exterior_values(c);
    return 1;
}
int boundary_rows(ak_case *c, std::vector<int32_t> &rows) {
    const long long n = c->nouter;
    std::vector<int> x(n), y(n), z(n);
    std::vector<signed char> d(n);
    if (n) {
        AK_CUDA(cudaMemcpy(x.data(), c->ox_, n * sizeof(int), cudaMemcpyDeviceToHost));
        AK_CUDA(cudaMemcpy(y.data(), c->oy_, n * sizeof(int), cudaMemcpyDeviceToHost));
        AK_CUDA(cudaMemcpy(z.data(), c->oz_, n * sizeof(int), cudaMemcpyDeviceToHost));
        AK_CUDA(cudaMemcpy(d.data(), c->od, n * sizeof(signed char), cudaMemcpyDeviceToHost));
    }
    rows.resize(4 * n);
    for (long long k = 0; k < n; ++k) {
        rows[4 * k] = x[k] - 1;
        rows[4 * k + 1] = y[k] - 1;
        rows[4 * k + 2] = z[k];
        rows[4 * k + 3] = d[k];
    }
    return AK_OK;
}
}  // namespace

int ak_boundary_state_size(ak_case *c, int64_t *n_links, int64_t *n_values) {
    AK_TRY(check_case(c));
    if (!n_links || !n_values) return fail(AK_ERR_INVALID, "null output");
    *n_links = c->nouter;
    *n_values = boundary_values(c);
    return AK_OK;
}

int ak_get_boundary_state(ak_case *c, int32_t *rows, double *values) {
    AK_TRY(check_case(c));
    if ((!rows && c->nouter) || !values) return fail(AK_ERR_INVALID, "null output");
    AK_CUDA(cudaStreamSynchronize(c->stream));
    std::vector<int32_t> r;
    AK_TRY(boundary_rows(c, r));
    if (!r.empty()) std::memcpy(rows, r.data(), r.size() * sizeof(int32_t));
    values[0] = c->prepared ? 1.0 : 0.0;
    double *v = values + 1;
    const long long n = c->nouter;
    if (c->farfield == AK_FARFIELD_CHARACTERISTIC) {
        std::vector<long long> clock(n);
        if (n) {
            AK_CUDA(cudaMemcpy(v, c->ff_in, n * sizeof(double), cudaMemcpyDeviceToHost));
            AK_CUDA(cudaMemcpy(v + n, c->ff_der, n * sizeof(double), cudaMemcpyDeviceToHost));
            AK_CUDA(cudaMemcpy(clock.data(), c->ff_clock, n * sizeof(long long), cudaMemcpyDeviceToHost));
        }
        for (long long k = 0; k < n; ++k) v[2 * n + k] = (double)clock[k];
        const long long rows_n = (long long)c->nx * c->nz;
        AK_CUDA(cudaMemcpy(v + 3 * n, c->ff_lo, rows_n * sizeof(double), cudaMemcpyDeviceToHost));
        AK_CUDA(cudaMemcpy(v + 3 * n + rows_n, c->ff_hi, rows_n * sizeof(double), cudaMemcpyDeviceToHost));
    } else if (c->farfield == AK_FARFIELD_LEGACY && c->n_out) {
        AK_CUDA(cudaMemcpy(v, c->out_state, 2 * c->n_out * sizeof(double), cudaMemcpyDeviceToHost));
    } else if (c->farfield == AK_FARFIELD_EXTERIOR) {
        AK_TRY(exterior_state(c, v, false));
    }
    return AK_OK;
}

int ak_set_boundary_state(ak_case *c, const int32_t *rows, const double *values) {
    AK_TRY(check_case(c));
    if ((!rows && c->nouter) || !values) return fail(AK_ERR_INVALID, "null input");
    AK_CUDA(cudaStreamSynchronize(c->stream));
    std::vector<int32_t> r;
    AK_TRY(boundary_rows(c, r));
    if (!r.empty() && std::memcmp(rows, r.data(), r.size() * sizeof(int32_t)) != 0)
        return fail(AK_ERR_INVALID, "boundary link geometry differs from this case's");
    const double *v = values + 1;
    const long long n = c->nouter;
    if (c->farfield == AK_FARFIELD_CHARACTERISTIC) {
        std::vector<long long> clock(n);
        for (long long k = 0; k < n; ++k) {
            const double t = v[2 * n + k];
            if (!(t >= 0.0) || t != std::floor(t)) return fail(AK_ERR_INVALID, "invalid glancing clock");
            clock[k] = (long long)t;
        }
        if (n) {
            AK_CUDA(cudaMemcpy(c->ff_in, v, n * sizeof(double), cudaMemcpyHostToDevice));
            AK_CUDA(cudaMemcpy(c->ff_der, v + n, n * sizeof(double), cudaMemcpyHostToDevice));
            AK_CUDA(cudaMemcpy(c->ff_clock, clock.data(), n * sizeof(long long), cudaMemcpyHostToDevice));
        }
        const long long rows_n = (long long)c->nx * c->nz;
        AK_CUDA(cudaMemcpy(c->ff_lo, v + 3 * n, rows_n * sizeof(double), cudaMemcpyHostToDevice));
        AK_CUDA(cudaMemcpy(c->ff_hi, v + 3 * n + rows_n, rows_n * sizeof(double), cudaMemcpyHostToDevice));
    } else if (c->farfield == AK_FARFIELD_LEGACY && c->n_out) {
        AK_CUDA(cudaMemcpy(c->out_state, v, 2 * c->n_out * sizeof(double), cudaMemcpyHostToDevice));
    } else if (c->farfield == AK_FARFIELD_EXTERIOR) {
        if (values[0] == 0.0) return fail(AK_ERR_INVALID, "an exterior checkpoint holds a prepared state");
        AK_TRY(exterior_state(c, const_cast<double *>(v), true));
    }
    c->prepared = values[0] != 0.0;
    return AK_OK;
}

int ak_exterior_report(ak_case *c, double *out) {
    AK_TRY(check_case(c));
    if (!out) return fail(AK_ERR_INVALID, "null output");
    if (c->farfield != AK_FARFIELD_EXTERIOR) return fail(AK_ERR_INVALID, "not an exterior case");
    AK_CUDA(cudaMemcpyAsync(out, c->ext_out, 11 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    AK_CUDA(cudaStreamSynchronize(c->stream));
    return AK_OK;
}

int ak_case_buffers(ak_case *c, void **current, void **other, int64_t *dims, int32_t *element_bytes) {
    AK_TRY(check_case(c));
    if (!current || !other || !dims || !element_bytes) return fail(AK_ERR_INVALID, "null output");
    AK_CUDA(cudaStreamSynchronize(c->stream));
    *current = c->pdf[c->cur];
    *other = c->pdf[1 - c->cur];
    dims[0] = Q;
    dims[1] = c->nz;
    dims[2] = c->G.nyp;
    dims[3] = c->G.sx;
    *element_bytes = (int32_t)c->esize;
    return AK_OK;
}

int ak_set_steps_done(ak_case *c, int64_t steps) {
    AK_TRY(check_case(c));
    if (steps < 0) return fail(AK_ERR_INVALID, "steps must be >= 0");
    c->steps = steps;
    if (c->farfield == AK_FARFIELD_EXTERIOR) {
        // the exterior step's clock (the traced incoming invariant's time)
        const double clock = (double)steps;
        AK_CUDA(cudaMemcpyAsync(c->ext_out + 11, &clock, sizeof(double), cudaMemcpyHostToDevice, c->stream));
        AK_CUDA(cudaStreamSynchronize(c->stream));
    }
    return AK_OK;
}

// ---- stationarity residuals (convergence.py:58-176) on the device
namespace {
long long residual_cells(const ak_case *c) {
    const int *r = c->res_region;
    return (long long)(r[1] - r[0]) * (r[3] - r[2]) * c->nz;
}
int ensure_residual_buffers(ak_case *c) {
    if (!c->res_snapshot) {
        AK_TRY(dalloc(c, &c->res_snapshot, (size_t)(4 * residual_cells(c))));
        AK_TRY(dalloc(c, &c->res_partials, (size_t)STATS_BLOCKS_CASE * 9));
        AK_TRY(dalloc(c, &c->res_out, 9));
    }
    return AK_OK;
}
}  // namespace

int ak_residuals(ak_case *c, double inv_speed, double inv_dt, int32_t reset, double *out) {
    AK_TRY(check_case(c));
    if (!out || !(inv_speed > 0) || !(inv_dt > 0)) return fail(AK_ERR_INVALID, "positive scales and an output are required");
    AK_TRY(ensure_residual_buffers(c));
    const int *g = c->res_region;
    const Region region{g[0], g[1], g[2], g[3], g[4], g[5], g[6], g[7]};
    AK_TRY(with_storage(c, [&](auto *tag) {
        using S = std::remove_pointer_t<decltype(tag)>;
        k_residuals<S><<<STATS_BLOCKS_CASE, 256, 0, c->stream>>>(src_of<S>(c), c->G, c->flags, region,
                                                                  c->res_snapshot, inv_speed, inv_dt, reset ? 1 : 0,
                                                                  c->res_partials);
        k_residuals_final<<<1, REDUCE_THREADS, 0, c->stream>>>(c->res_partials, STATS_BLOCKS_CASE, c->res_out);
        AK_CUDA(cudaGetLastError());
        return AK_OK;
    }));
    AK_CUDA(cudaMemcpyAsync(out, c->res_out, 9 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    AK_CUDA(cudaStreamSynchronize(c->stream));
    return AK_OK;
}

int ak_residual_snapshot(ak_case *c, int32_t write, double *data, int64_t *count) {
    AK_TRY(check_case(c));
    if (!count) return fail(AK_ERR_INVALID, "null count");
    *count = 4 * residual_cells(c);
    if (!data) return AK_OK;
    AK_TRY(ensure_residual_buffers(c));
    AK_CUDA(cudaStreamSynchronize(c->stream));
    if (write)
        AK_CUDA(cudaMemcpy(c->res_snapshot, data, *count * sizeof(double), cudaMemcpyHostToDevice));
    else
        AK_CUDA(cudaMemcpy(data, c->res_snapshot, *count * sizeof(double), cudaMemcpyDeviceToHost));
    return AK_OK;
}

int ak_get_flags(ak_case *c, uint8_t *flags) {
    AK_TRY(check_case(c));
    if (!flags) return fail(AK_ERR_INVALID, "null output");
    const int nxp = c->nx + 2;
    std::vector<uint8_t> h((size_t)nxp * (c->ny + 2));
    AK_CUDA(cudaMemcpyAsync(h.data(), c->flags, h.size(), cudaMemcpyDeviceToHost, c->stream));
    AK_CUDA(cudaStreamSynchronize(c->stream));
    for (int x = 0; x < c->nx; ++x)
        for (int y = 0; y < c->ny; ++y) flags[(size_t)x * c->ny + y] = h[(size_t)(y + 1) * nxp + (x + 1)];
    return AK_OK;
}

int ak_get_wall_links(ak_case *c, int32_t *rows, double *q) {
    AK_TRY(check_case(c));
    if ((!rows || !q) && c->nkeys) return fail(AK_ERR_INVALID, "null output");
    std::vector<WallKey> keys((size_t)c->nkeys);
    if (c->nkeys) {
        AK_CUDA(cudaMemcpyAsync(keys.data(), c->keys, keys.size() * sizeof(WallKey), cudaMemcpyDeviceToHost, c->stream));
        AK_CUDA(cudaMemcpyAsync(q, c->wall_q, c->nkeys * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    }
    AK_CUDA(cudaStreamSynchronize(c->stream));
    for (long long k = 0; k < c->nkeys; ++k) {
        rows[4 * k] = keys[k].element;
        rows[4 * k + 1] = keys[k].x - 1;
        rows[4 * k + 2] = keys[k].y - 1;
        rows[4 * k + 3] = keys[k].d2;
    }
    return AK_OK;
}

}  // extern "C"

// ==================================================================== refined
// Two-level 2:1 case (refined_solver.py:115-345, interface.py:133-352): a
// coarse lattice with the legacy outer boundary and a padded fine block with
// the walls, advanced as one coarse step + two fine steps per call, with
// time-interpolated donors, face-flux reflux and restriction.  Every kernel
// of a refined case runs on the coarse lattice's stream.
struct ak_refined {
    ak_case *coarse = nullptr, *fine = nullptr;
    BoxSpec B{};
    int pad = 2;
    // The coarse level keeps post-collision populations outside the transfer
    // block (the box and three coarse cells around it, padded coordinates
    // x [xfer.x, xfer.y) by y [xfer.z, xfer.w)), whose cells the donors read
    // and the reflux and restriction write as pre-collision populations
    // there: the coarse streaming of one step then fuses with the next
    // step's collision everywhere else.  Used when the block lies inside the
    // lattice (the donor block does not wrap).
    bool fused = false;
    int4 xfer{0, 0, 0, 0};
    // where the reference's pre-collision coarse state lives (fused form):
    // 0 the other copy holds it (after set-up), 1 it is the other copy pulled
    // (after a step: the fused pass read that copy, boundaries applied, and
    // collided what it pulled), -1 unknown; valid while the coarse level's
    // pdf_writes equals pre_writes
    int pre_mode = -1;
    long long pre_writes = 0;
    // the outer boundaries' branch inside the captured graphs (fused form,
    // transfer block at least three columns from every outer face): UBB,
    // outflow and the budget's outer flux run beside the transfer-block
    // collision, whose cells they neither read nor write
    // The same branch then streams and collides the coarse cells outside
    // near (the transfer block and one cell around it, padded coordinates):
    // they pull only from cells outside the block, which nothing in the step
    // writes, so the pass runs beside the rest of the step (the second fine
    // step, restriction, reflux) at the least priority, and the step's own
    // stream takes the cells of near alone.
    bool bnd_branch = false;
    int4 near{0, 0, 0, 0};
    cudaStream_t bnd = nullptr;
    cudaEvent_t ev_bnd_in = nullptr, ev_bnd_out = nullptr;
    // two steps in one captured graph: the first leaves its far pass (and
    // the budget's reduction of its rows) open on the boundaries' branch, and
    // the second's near pass waits for it (ev_far_done); ev_band_done orders
    // that reduction after the band's sums
    cudaEvent_t ev_far_done = nullptr, ev_band_done = nullptr;
    // the budget's outer-face flux beside the far pass: it reads the coarse
    // copy (ghosts written by UBB and outflow), which the far pass only reads
    cudaStream_t ostr = nullptr;
    cudaEvent_t ev_outer_in = nullptr, ev_outer_out = nullptr;
    double dx_c = 0, dt_c = 0, dx_f = 0, dt_f = 0, span = 0, speed = 0;
    double tau_s_c = 0, tau_b_c = 0, tau_s_f = 0, tau_b_f = 0;
    double free_g[Q];
    double *d_free = nullptr;
    double *mom_old = nullptr, *mom_new = nullptr, *mom_half = nullptr;
    double *pro_x = nullptr;  // donor moments after the x prolongation pass (first fine step)
    double *pro_x2 = nullptr; // the same for the second fine step, made right after the coarse step
    Face faces[4];
    int nfaces = 0;
    long long offs[4] = {0, 0, 0, 0};
    long long reg_doubles = 0, max_face = 0;
    Face *d_faces = nullptr;
    long long *d_offs = nullptr;
    double *reg_c = nullptr, *reg_f = nullptr;
    FluxTerm *d_terms[2] = {nullptr, nullptr};
    int nterms = 0;
    int *d_flag = nullptr;
    double *d_loads = nullptr;
    // the step's report in one device block, copied to the host at once:
    // validity flag (an int in the first slot), both fine steps' loads,
    // outer-face flux (outer_out), integrals (stats_out); a pinned copy
    double *report = nullptr, *host_report = nullptr;
    long long report_doubles = 0;
    unsigned *wall_done = nullptr;  // finished-block counters of the two fine steps' wall launches
    unsigned *rows_done = nullptr;  // the same for the coarse and the fine budget rows' reductions
    long long steps = 0;
    std::vector<void *> owned;  // device buffers the two-level case owns
    // one captured coarse step (or two) per (coarse, fine) buffer parity,
    // replayed by ak_refined_step; graph_launches counts the kernels of one
    // replay
    // (coarse copy, fine copy, budget, step integrals) x (1, 2 or 4 steps)
    cudaGraphExec_t graph[48] = {};
    long long graph_launches[48] = {};
    bool step_stats = false;         // the step ends with the budget's integrals
    cudaStream_t side = nullptr;  // the first fine step's stream inside the captured graphs
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // the face-flux registers' branch inside the captured graphs: the coarse
    // and both fine face fluxes run in order on their own stream beside the
    // boundaries, walls and streaming, and join before the reflux
    cudaStream_t flux = nullptr;
    cudaEvent_t ev_flux_in[3] = {nullptr, nullptr, nullptr}, ev_flux_f0 = nullptr, ev_flux_done = nullptr;
    // budget support: inflow through the outer x/y faces of each tracked step,
    // and the per-level statistics of the conserved integrals / validity check
    bool track_budget = false;
    Face outer[4];
    Face *d_outer = nullptr;
    int outer_blocks = 0;
    double *outer_partials = nullptr, *outer_out = nullptr;  // outer_out: last step [4], running sum [4]
    double *cum_loads = nullptr;                              // wall loads summed over all steps [n * 5]
    double *stats_partials = nullptr, *stats_out = nullptr;
    long long *fine_rows = nullptr;  // the fine block's budget rows
    double *fine_stage = nullptr;
    // fused form in an FP64-arithmetic storage: the coarse statistics of a
    // budget step come from the fused pass itself (rows of its far and near
    // launches, then the transfer block's band outside the box)
    long long *cstats = nullptr;  // budget rows (warp_budget_row)
    double *cstats_stage = nullptr;
    long long cstats_far = 0, cstats_near = 0;
};

namespace {

template <typename T>
int ralloc(ak_refined *R, T **p, size_t n) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess)
        return fail(e == cudaErrorMemoryAllocation ? AK_ERR_NOMEM : AK_ERR_CUDA,
                    std::string("device allocation failed: ") + cudaGetErrorString(e));
    R->owned.push_back(*p);
    return AK_OK;
}

void refined_release(ak_refined *R) {
    if (R->coarse) cudaStreamSynchronize(R->coarse->stream);
    for (cudaGraphExec_t &g : R->graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    for (void *p : R->owned) cudaFree(p);
    if (R->host_report) cudaFreeHost(R->host_report);
    if (R->ev_fork) cudaEventDestroy(R->ev_fork);
    if (R->ev_join) cudaEventDestroy(R->ev_join);
    if (R->side) cudaStreamDestroy(R->side);
    for (cudaEvent_t e : {R->ev_flux_in[0], R->ev_flux_in[1], R->ev_flux_in[2], R->ev_flux_f0, R->ev_flux_done})
        if (e) cudaEventDestroy(e);
    if (R->flux) cudaStreamDestroy(R->flux);
    if (R->ev_bnd_in) cudaEventDestroy(R->ev_bnd_in);
    if (R->ev_outer_in) cudaEventDestroy(R->ev_outer_in);
    if (R->ev_outer_out) cudaEventDestroy(R->ev_outer_out);
    if (R->ostr) cudaStreamDestroy(R->ostr);
    if (R->ev_bnd_out) cudaEventDestroy(R->ev_bnd_out);
    if (R->ev_far_done) cudaEventDestroy(R->ev_far_done);
    if (R->ev_band_done) cudaEventDestroy(R->ev_band_done);
    if (R->bnd) cudaStreamDestroy(R->bnd);
    if (R->coarse) {
        release(R->coarse);
        delete R->coarse;
    }
    if (R->fine) {
        release(R->fine);
        delete R->fine;
    }
}

// zero-centred populations of (rho = 1, u = (U, 0, 0)) with zero stress
void free_populations(double speed, double g[Q]) {
    for (int q = 0; q < Q; ++q) {
        const int c[3] = {cx(q), cy(q), cz(q)};
        const double u[3] = {speed, 0.0, 0.0};
        double eq = 1.0;
        for (int a = 0; a < 3; ++a)
            eq *= c[a] == 0 ? 2.0 / 3.0 - u[a] * u[a] : (1.0 / 3.0 + u[a] * u[a] + c[a] * u[a]) / 2.0;
        g[q] = eq - weight(q);
    }
}

// face-flux terms of one normal axis (interface.py:73-94)
std::vector<FluxTerm> flux_terms(int axis) {
    std::vector<FluxTerm> out;
    for (int d = 0; d < Q; ++d) {
        const int c[3] = {cx(d), cy(d), cz(d)};
        const int normal = c[axis];
        if (normal == 0) continue;
        std::vector<int> moving;
        for (int a = 0; a < 3; ++a)
            if (a != axis && c[a] != 0) moving.push_back(a);
        const int m = (int)moving.size();
        auto fact = [](int n) { double f = 1; for (int k = 2; k <= n; ++k) f *= k; return f; };
        for (int count = 0; count <= m; ++count) {
            const double weight_ = fact(count) * fact(m - count) / fact(m + 1);
            for (int mask = 0; mask < (1 << m); ++mask) {
                if (__builtin_popcount(mask) != count) continue;
                FluxTerm t{};
                t.d = d;
                for (int k = 0; k < m; ++k)
                    if (mask & (1 << k)) t.shift[moving[k]] = -c[moving[k]];
                t.coef[0] = weight_ * normal;
                for (int a = 0; a < 3; ++a) t.coef[a + 1] = weight_ * normal * c[a];
                out.push_back(t);
            }
        }
    }
    return out;
}

long long blocks3(long long n) { return (n + 255) / 256; }
// fixed grid of the region statistics (results do not depend on the device)
constexpr int STATS_BLOCKS = 4 * 152;
// direction-split kernels: 32 cells per 256-thread block
long long split_blocks(long long cells) { return (cells + SPLIT_CELLS - 1) / SPLIT_CELLS; }

// dispatch on the storage pair of a two-level case: both levels in one form,
// or the FP16 form's FP32 fine level (the walls' level)
template <typename F>
int with_levels(ak_refined *R, F &&f) {
    const int c = R->coarse->storage, fs = R->fine->storage;
    if (c == fs) return with_storage(R->coarse, [&](auto *tag) { return f(tag, tag); });
    if (c == AK_STORAGE_F16 && fs == AK_STORAGE_F32) return f((__half *)nullptr, (float *)nullptr);
    return fail(AK_ERR_INVALID, "unsupported pair of level storage forms");
}
#define AK_LEVEL_TYPES(a, b) using S = std::remove_pointer_t<decltype(a)>; using SF = std::remove_pointer_t<decltype(b)>
// a donor-moment buffer (allocated as doubles) in the transfer arithmetic
// type of the coarse storage S (FP32 for the FP32-compute forms)
template <typename S>
typename Store<S>::A *moments_of(double *p) {
    return reinterpret_cast<typename Store<S>::A *>(p);
}

// restriction of the fine block onto the covered coarse cells
template <typename S, typename SF>
cudaError_t launch_restrict(ak_refined *R, const Rescale &f2c, cudaStream_t st) {
    const BoxSpec &B = R->B;
    const long long ring = ring_count(B.bx, B.by, 3, 3) * B.bz;
    const long long core = (long long)std::max(B.bx - 6, 0) * std::max(B.by - 6, 0) * B.bz;
    const long long nb = std::max(split_blocks(ring), blocks3(core));
    return launch_chained(CHAIN_TAIL, k_restrict<S, SF>, dim3((unsigned)nb, 2), dim3(SPLIT_THREADS), st, src_of<S>(R->coarse),
                   R->coarse->G, (const SF *)src_of<SF>(R->fine), R->fine->G, B, R->pad, (const double *)R->d_free, f2c,
                   R->d_flag);
}

template <typename S, typename SF>
int refined_init(ak_refined *R, double amp, double phase_y, double phase_z, double lead_x, double lead_y) {
    ak_case *C = R->coarse, *F = R->fine;
    cudaStream_t st = C->stream;
    const double ky = 2 * M_PI / (C->ny * R->dx_c), kz = 2 * M_PI / R->span;
    // both copies of a level at the free stream, then the perturbed state
    auto level = [&](ak_case *L, auto *tag) -> int {
        using SL = std::remove_pointer_t<decltype(tag)>;
        for (int k = 0; k < 2; ++k)
            k_fill<SL><<<(unsigned)blocks3(L->G.qs), 256, 0, st>>>((SL *)L->pdf[k], L->G, R->d_free);
        const long long n = (long long)L->nx * L->ny * L->nz;
        k_init_perturbed<SL><<<(unsigned)blocks3(n), 256, 0, st>>>(src_of<SL>(L), L->G, L->flags, R->speed, amp,
                                                                    phase_y, phase_z, lead_x, lead_y, L->origin_x,
                                                                    L->origin_y, L->dx, ky, kz);
        AK_CUDA(cudaGetLastError());
        return AK_OK;
    };
    AK_TRY(level(C, (S *)nullptr));
    AK_TRY(level(F, (SF *)nullptr));
    const Rescale f2c{R->tau_s_c * R->dt_c / (R->tau_s_f * R->dt_f), R->tau_b_c * R->dt_c / (R->tau_b_f * R->dt_f)};
    AK_CUDA(cudaMemsetAsync(R->d_flag, 0, sizeof(int), st));
    AK_CUDA((launch_restrict<S, SF>(R, f2c, st)));
    AK_CUDA(cudaGetLastError());
    // boundary data from the initial state, ghosts still holding the free
    // stream (refined_solver.py:224-262)
    if (C->n_out) {
        k_outflow_prepare<S><<<(unsigned)blocks3(C->n_out), 256, 0, st>>>(
            src_of<S>(C), C->G, C->outer(), C->sel_out, C->n_out, C->out_state, 1, 0, 0, 1.0, C->speed, 0.0, 0.0);
        AK_CUDA(cudaGetLastError());
    }
    if (R->fused) {
        // outside the transfer block the coarse level stores post-collision;
        // the other copy keeps the pre-collision state until the first step
        // writes it
        using T = typename Store<S>::T;
        AK_CUDA(cudaMemcpyAsync(dst_of<S>(C), src_of<S>(C), sizeof(S) * (size_t)Q * C->G.qs,
                                cudaMemcpyDeviceToDevice, st));
        R->pre_mode = 0;
        R->pre_writes = C->pdf_writes;
        k_collide<S><<<(unsigned)blocks_for((long long)C->nx * C->ny * C->nz, 128), 128, 0, st>>>(
            src_of<S>(C), C->flags, C->G, C->shift_host, (T)C->omega_s, (T)C->omega_b, make_int4(0, 0, 0, 0),
            R->xfer);
        AK_CUDA(cudaGetLastError());
    }
    C->prepared = F->prepared = true;
    R->steps = 0;
    AK_CUDA(cudaMemsetAsync(R->outer_out, 0, 8 * sizeof(double), st));
    AK_CUDA(cudaMemsetAsync(R->cum_loads, 0, 5 * std::max(1, F->n_elements) * sizeof(double), st));
    AK_CUDA(cudaStreamSynchronize(st));
    int flag = 0;
    AK_CUDA(cudaMemcpy(&flag, R->d_flag, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) return fail(AK_ERR_NONFINITE, "initial restriction produced an invalid state");
    return AK_OK;
}

// Mass, momentum and validity statistics of the coarse cells outside the
// fine box and the fine block's physical cells, into stats_out[2][NSTAT]
// (refined_solver.py:291-299, 347-361).
// the storage forms whose collision arithmetic is FP64-accurate: their fused
// pass supplies the budget's coarse mass and momentum sums
template <typename S>
__host__ __device__ constexpr bool fused_stats_form() {
    return std::is_same_v<S, double> || std::is_same_v<S, df2>;
}

// reduction of budget rows into out[NSTAT]: one block when they are few,
// else a first stage into stage (blocks_for(nrows, REDUCE_THREADS) rows)
int enqueue_rows_final(ak_refined *R, const long long *rows, long long nrows, double *stage, unsigned *done,
                       double *out, cudaStream_t st) {
    if (nrows <= 16 * REDUCE_THREADS) {
        k_budget_final<<<1, REDUCE_THREADS, 0, st>>>(rows, nrows, out);
    } else {
        // one launch: its last block to finish reduces the stage
        const long long ns = blocks_for(nrows, REDUCE_THREADS);
        k_budget_stage<<<(unsigned)ns, REDUCE_THREADS, 0, st>>>(rows, nrows, stage, done, out);
    }
    R->coarse->launches += 1;
    AK_CUDA(cudaGetLastError());
    return AK_OK;
}

// the fine block's physical cells (interior coordinates of the padded block)
Region fine_region(const ak_refined *R) {
    const ak_case *F = R->fine;
    return Region{R->pad, F->nx - R->pad, R->pad, F->ny - R->pad, 0, 0, 0, 0};
}
long long region_cells(const Region &g, int nz) { return (long long)(g.x1 - g.x0) * (g.y1 - g.y0) * nz; }

// The fine block's budget sums (stats_out[NSTAT..2 NSTAT)), on the stream
// the restriction runs on: both only read the fine state.
template <typename SF>
int enqueue_fine_stats(ak_refined *R, cudaStream_t st) {
    ak_case *F = R->fine;
    const Region rf = fine_region(R);
    const long long rows = region_sum_rows(region_cells(rf, F->nz));
    AK_CUDA(launch_chained(CHAIN_TAIL, k_region_sums<SF>, dim3((unsigned)(rows / 8)), dim3(256), st, (const SF *)src_of<SF>(F),
                           F->G, (const uint8_t *)F->flags, rf, R->fine_rows));
    R->coarse->launches += 1;
    AK_CUDA(cudaGetLastError());
    return enqueue_rows_final(R, R->fine_rows, rows, R->fine_stage, R->rows_done + 1, R->stats_out + NSTAT, st);
}

// The coarse budget sums when the fused coarse pass has written its rows to
// cstats: the cells of the transfer block outside the box (after reflux and
// restriction), then the reduction over every row.
Region band_region(const ak_refined *R) {
    const BoxSpec &B = R->B;
    return Region{R->xfer.x - 1, R->xfer.y - 1, R->xfer.z - 1, R->xfer.w - 1, B.lo[0], B.hi[0], B.lo[1], B.hi[1]};
}
// the band's rows, as soon as its cells are final (after the reflux)
template <typename S>
int enqueue_band_sums(ak_refined *R, cudaStream_t st) {
    ak_case *C = R->coarse;
    const Region band = band_region(R);
    const long long band_rows = region_sum_rows(region_cells(band, C->nz));
    AK_CUDA(launch_chained(CHAIN_TAIL, k_region_sums<S>, dim3((unsigned)(band_rows / 8)), dim3(256), st, (const S *)src_of<S>(C),
                           C->G, (const uint8_t *)C->flags, band,
                           R->cstats + (R->cstats_far + R->cstats_near) * NSTAT));
    C->launches += 1;
    AK_CUDA(cudaGetLastError());
    return AK_OK;
}
// every coarse row into stats_out[0..NSTAT), once the fused pass has ended
int enqueue_coarse_rows_final(ak_refined *R, cudaStream_t st) {
    const long long band_rows = region_sum_rows(region_cells(band_region(R), R->coarse->nz));
    return enqueue_rows_final(R, R->cstats, R->cstats_far + R->cstats_near + band_rows, R->cstats_stage,
                              R->rows_done, R->stats_out, st);
}

template <typename S, typename SF>
int enqueue_region_stats(ak_refined *R, cudaStream_t st) {
    ak_case *C = R->coarse, *F = R->fine;
    const BoxSpec &B = R->B;
    const Region rc{0, C->nx, 0, C->ny, B.lo[0], B.hi[0], B.lo[1], B.hi[1]};
    const Region rf{R->pad, F->nx - R->pad, R->pad, F->ny - R->pad, 0, 0, 0, 0};
    k_region_stats<S><<<STATS_BLOCKS, 256, 0, st>>>(src_of<S>(C), C->G, C->flags, rc, R->stats_partials);
    k_region_final<<<1, REDUCE_THREADS, 0, st>>>(R->stats_partials, STATS_BLOCKS, R->stats_out);
    k_region_stats<SF><<<STATS_BLOCKS, 256, 0, st>>>(src_of<SF>(F), F->G, F->flags, rf, R->stats_partials);
    k_region_final<<<1, REDUCE_THREADS, 0, st>>>(R->stats_partials, STATS_BLOCKS, R->stats_out + NSTAT);
    C->launches += 4;
    AK_CUDA(cudaGetLastError());
    return AK_OK;
}

// after_open: the previous step of the same capture left its far pass open
// (leave_open); this step's near pass waits for it.  Both need fork mode
// with the boundaries' branch.
template <typename S, typename SF>
int refined_step(ak_refined *R, bool fork = false, bool after_open = false, bool leave_open = false) {
    using T = typename Store<S>::T;
    using TF = typename Store<SF>::T;
    ak_case *C = R->coarse, *F = R->fine;
    cudaStream_t st = C->stream;
    const BoxSpec &B = R->B;
    const long long nring_block = ring_count(B.dnx, B.dny, DONOR_RING, DONOR_RING) * C->nz;
    dim3 gc((unsigned)blocks_for(C->nx, 128), (unsigned)C->ny, (unsigned)C->nz);
    dim3 gf((unsigned)blocks_for(F->nx, 128), (unsigned)F->ny, (unsigned)F->nz);
    // the collisions number their cells across rows (1-D grids)
    const unsigned gc1 = (unsigned)blocks_for((long long)C->nx * C->ny * C->nz, 128);
    const unsigned gx1 = (unsigned)blocks_for((long long)(R->xfer.y - R->xfer.x) * (R->xfer.w - R->xfer.z) * C->nz, 128);
    // the stream-collide's grids (cells, or cell pairs in the pair forms):
    // the whole lattice and the near part
    const unsigned gsc = stream_collide_grid<S>(make_int4(0, 0, 0, 0), C->nx, C->ny, C->nz);
    const unsigned gsn = stream_collide_grid<S>(R->near, C->nx, C->ny, C->nz);
    // fork mode, fused form, transfer block away from the outer faces: the
    // boundaries and the far coarse pass on their own branch
    const bool bnd = fork && R->fused && R->bnd_branch;
    // a budget step of an FP64-arithmetic fused form takes its coarse
    // statistics from the fused pass
    bool fstats = false;
    if constexpr (fused_stats_form<S>()) fstats = R->track_budget && R->step_stats && R->fused && R->cstats;
    const unsigned gf1 = (unsigned)blocks_for((long long)F->nx * F->ny * F->nz, 128);
    const Rescale c2f{R->tau_s_f * R->dt_f / (R->tau_s_c * R->dt_c), R->tau_b_f * R->dt_f / (R->tau_b_c * R->dt_c)};
    const Rescale f2c{R->tau_s_c * R->dt_c / (R->tau_s_f * R->dt_f), R->tau_b_c * R->dt_c / (R->tau_b_f * R->dt_f)};
    const long long nband = ring_count(F->nx, F->ny, R->pad, R->pad) * F->nz;
    const long long nprox = ring_count(F->nx, B.dny, R->pad, DONOR_RING) * C->nz;
    const long long nlinks = F->nkeys * F->nz * 3;
    const long long nb = blocks_for(nlinks, 256);

    // the stream a face flux runs on: in the captured graph the flux branch,
    // entered after the collision on stream s (slot: 0 coarse, 1 + sub fine)
    auto flux_stream = [&](cudaStream_t s, int slot) -> cudaStream_t {
        if (!fork) return s;
        if (cudaEventRecord(R->ev_flux_in[slot], s) != cudaSuccess ||
            cudaStreamWaitEvent(R->flux, R->ev_flux_in[slot], 0) != cudaSuccess)
            return nullptr;
        return R->flux;
    };
    // the outer boundaries of the coarse level on stream s: UBB, outflow and
    // the budget's flux through the outer faces
    // in the boundaries' branch (bnd) the budget's flux forks onto its own
    // stream, so that the far pass does not wait for it
    auto outer_part = [&](cudaStream_t s) -> int {
        if (C->n_ubb)
            k_ubb<S><<<(unsigned)blocks3(C->n_ubb_cells * C->nz), 256, 0, s>>>(src_of<S>(C), C->G, C->ubb_cells,
                                                                               C->n_ubb_cells, C->speed, 0.0, 0.0);
        if (C->n_out)
            k_outflow<S><<<(unsigned)blocks3(C->n_out), 256, 0, s>>>(src_of<S>(C), C->G, C->outer(), C->sel_out,
                                                                     C->n_out, C->out_state, 1, 0, 0);
        if (R->track_budget) {
            cudaStream_t fs = s;
            if (bnd) {
                AK_CUDA(cudaEventRecord(R->ev_outer_in, s));
                AK_CUDA(cudaStreamWaitEvent(R->ostr, R->ev_outer_in, 0));
                fs = R->ostr;
            }
            k_outer_flux<S><<<dim3((unsigned)R->outer_blocks, 4), 256, 0, fs>>>(
                src_of<S>(C), C->G, R->d_terms[0], R->d_terms[1], R->nterms, R->d_outer, 4, R->outer_partials);
            k_outer_final<<<1, REDUCE_THREADS, 0, fs>>>(R->outer_partials, R->d_outer, 4, R->outer_blocks,
                                                       R->dx_c * R->dx_c * R->dx_c, R->outer_out);
            if (bnd) AK_CUDA(cudaEventRecord(R->ev_outer_out, fs));
            C->launches += 2;
        }
        AK_CUDA(cudaGetLastError());
        return AK_OK;
    };
    // coarse collide, face fluxes, outer boundary, stream, donors after the step
    auto coarse_part = [&]() -> int {
        if (bnd) {
            AK_CUDA(cudaEventRecord(R->ev_bnd_in, st));
            AK_CUDA(cudaStreamWaitEvent(R->bnd, R->ev_bnd_in, 0));
            AK_TRY(outer_part(R->bnd));
            if (fstats)
                k_stream_collide<S, true><<<gsc, 128, 0, R->bnd>>>(
                    src_of<S>(C), dst_of<S>(C), C->flags, C->G, C->shift_host, (T)C->omega_s, (T)C->omega_b,
                    Sgs<T>{}, R->xfer, make_int4(0, 0, 0, 0), R->near, R->cstats);
            else
                k_stream_collide<S><<<gsc, 128, 0, R->bnd>>>(src_of<S>(C), dst_of<S>(C), C->flags, C->G,
                                                              C->shift_host, (T)C->omega_s, (T)C->omega_b, Sgs<T>{},
                                                              R->xfer, make_int4(0, 0, 0, 0), R->near);
            AK_CUDA(cudaEventRecord(R->ev_bnd_out, R->bnd));
        }
        mark(C);
        // fused: only the transfer block holds pre-collision populations (a
        // grid over its cells alone)
        if (R->fused)
            AK_CUDA(launch_chained(CHAIN_COARSE, k_collide<S>, dim3(gx1), dim3(128), st, src_of<S>(C), C->flags, C->G,
                                   C->shift_host, (T)C->omega_s, (T)C->omega_b, R->xfer, make_int4(0, 0, 0, 0)));
        else
            k_collide<S><<<gc1, 128, 0, st>>>(src_of<S>(C), C->flags, C->G, C->shift_host, (T)C->omega_s,
                                              (T)C->omega_b);
        mark(C);
        cudaStream_t fs = flux_stream(st, 0);
        if (!fs) return fail(AK_ERR_CUDA, "face-flux branch could not be forked");
        // reads the post-collision coarse copy, which nothing in this step
        // writes afterwards (streaming writes the other copy)
        k_face_flux_coarse<S><<<dim3((unsigned)blocks3(32 * R->max_face), R->nfaces), 256, 0, fs>>>(
            src_of<S>(C), C->G, R->d_terms[0], R->d_terms[1], R->nterms, R->d_faces, R->nfaces, R->d_offs,
            R->dx_c * R->dx_c * R->dx_c, R->reg_c);
        if (!bnd) AK_TRY(outer_part(st));
        mark(C);
        // the near cells pull from cells the previous step's far pass wrote
        if (bnd && after_open) AK_CUDA(cudaStreamWaitEvent(st, R->ev_far_done, 0));
        if (bnd && fstats)
            AK_CUDA(launch_chained(CHAIN_COARSE, k_stream_collide<S, true>, dim3(gsn), dim3(128), st, (const S *)src_of<S>(C),
                                   dst_of<S>(C), (const uint8_t *)C->flags, C->G, C->shift_host, (T)C->omega_s,
                                   (T)C->omega_b, Sgs<T>{}, R->xfer, R->near, make_int4(0, 0, 0, 0),
                                   R->cstats + R->cstats_far * NSTAT));
        else if (bnd)
            // the cells of near; the rest runs on the boundaries' branch
            AK_CUDA(launch_chained(CHAIN_COARSE, k_stream_collide<S, false>, dim3(gsn), dim3(128), st, (const S *)src_of<S>(C),
                                   dst_of<S>(C), (const uint8_t *)C->flags, C->G, C->shift_host, (T)C->omega_s,
                                   (T)C->omega_b, Sgs<T>{}, R->xfer, R->near, make_int4(0, 0, 0, 0),
                                   (long long *)nullptr));
        else if (R->fused && fstats) {
            // one launch covers every row of the far part; the near rows stay empty
            AK_CUDA(cudaMemsetAsync(R->cstats + R->cstats_far * NSTAT, 0, sizeof(long long) * R->cstats_near * NSTAT, st));
            k_stream_collide<S, true><<<gsc, 128, 0, st>>>(src_of<S>(C), dst_of<S>(C), C->flags, C->G,
                                                            C->shift_host, (T)C->omega_s, (T)C->omega_b, Sgs<T>{},
                                                            R->xfer, make_int4(0, 0, 0, 0), make_int4(0, 0, 0, 0),
                                                            R->cstats);
        } else if (R->fused)
            // streaming fused with the next step's collision, the transfer
            // block streamed only
            k_stream_collide<S><<<gsc, 128, 0, st>>>(src_of<S>(C), dst_of<S>(C), C->flags, C->G, C->shift_host,
                                                      (T)C->omega_s, (T)C->omega_b, Sgs<T>{}, R->xfer);
        else
            k_stream<S><<<gc, 128, 0, st>>>(src_of<S>(C), dst_of<S>(C), C->flags, C->G, 0);
        mark(C);
        AK_CUDA(cudaGetLastError());
        C->cur = 1 - C->cur;
        AK_CUDA(launch_chained(CHAIN_COARSE, k_block_moments<S>, dim3((unsigned)split_blocks(nring_block)), dim3(SPLIT_THREADS), st,
                               (const S *)src_of<S>(C), C->G, B, (const double *)R->d_free, moments_of<S>(R->mom_new),
                               (const typename Store<S>::A *)moments_of<S>(R->mom_old), moments_of<S>(R->mom_half),
                               R->d_flag));
        // the second fine step's x pass, from the half-way donor moments: it
        // needs nothing of the first fine step, so it runs before the join
        AK_CUDA(launch_chained(CHAIN_PROLONG, k_prolong_x<typename Store<S>::A>, dim3((unsigned)blocks3(nprox)),
                               dim3(256), st, B, C->nz, R->pad, (const typename Store<S>::A *)moments_of<S>(R->mom_half),
                               moments_of<S>(R->pro_x2)));
        AK_CUDA(cudaGetLastError());
        return AK_OK;
    };
    // The fine steps, fused: the first fine step streams with the
    // collision of the second over the physical block (the band's cells are
    // overwritten by the second step's donors), and the second step collides
    // only the band.  In the FP32 fine storage the donor kernel collides the
    // band itself (its 32-cell blocks are cheap to collide in FP32; in the
    // FP64-arithmetic forms one warp per block would serialise the FP64
    // collision, and FP16 storage rounds the donors before the collision), in
    // the others a band-only collision follows the donors.  The fine state
    // between coarse steps stays pre-collision.
    constexpr bool fine_fused = true;
    constexpr bool donors_collide = fine_fused && std::is_same_v<SF, float>;
    const int4 fine_rect = make_int4(1 + R->pad, F->nx + 1 - R->pad, 1 + R->pad, F->ny + 1 - R->pad);
    const unsigned gfr = stream_collide_grid<SF>(fine_rect, F->nx, F->ny, F->nz);
    // one fine step on stream s: donors, collide, face fluxes, walls, stream
    auto fine_part = [&](int sub, cudaStream_t s) -> int {
        // donor moments at the fine step's start: the old coarse state, then
        // half-way (1 - 1/2) old + 1/2 new (refined_solver.py:311-318)
        // (the second fine step's x pass ran at the end of the coarse step)
        if (sub == 0)
            AK_CUDA(launch_chained(CHAIN_PROLONG, k_prolong_x<typename Store<S>::A>, dim3((unsigned)blocks3(nprox)),
                                   dim3(256), s, B, C->nz, R->pad,
                                   (const typename Store<S>::A *)moments_of<S>(R->mom_old), moments_of<S>(R->pro_x)));
        const typename Store<S>::A *px = moments_of<S>(sub ? R->pro_x2 : R->pro_x);
        bool collided = false;
        const dim3 gd((unsigned)split_blocks(nband)), bd(SPLIT_THREADS);
        if constexpr (donors_collide) {
            if (sub == 1) {
                AK_CUDA(launch_chained(CHAIN_FINE, k_donors<SF, true>, gd, bd, s, src_of<SF>(F), F->G, C->nz,
                                       px, B.dny, c2f, R->pad, R->d_flag, F->flags,
                                       (TF)F->omega_s, (TF)F->omega_b));
                collided = true;
            }
        }
        if (!collided)
            AK_CUDA(launch_chained(CHAIN_FINE, k_donors<SF, false>, gd, bd, s, src_of<SF>(F), F->G, C->nz, px,
                                   B.dny, c2f, R->pad, R->d_flag, (const uint8_t *)nullptr, (TF)0, (TF)0));
        mark(C);
        if (sub == 0 || !fine_fused)
            AK_CUDA(launch_chained(CHAIN_FINE, k_collide<SF>, dim3(gf1), dim3(128), s, src_of<SF>(F), F->flags, F->G,
                                   F->shift_host, (TF)F->omega_s, (TF)F->omega_b, make_int4(0, 0, 0, 0),
                                   make_int4(0, 0, 0, 0)));
        else if (!collided)
            // the band alone: the physical block was collided by the first
            // step's stream-collide
            AK_CUDA(launch_chained(CHAIN_FINE, k_collide_band<SF>, dim3((unsigned)blocks_for(nband, 128)), dim3(128), s,
                                   src_of<SF>(F), F->flags, F->G, F->shift_host, (TF)F->omega_s, (TF)F->omega_b,
                                   R->pad));
        mark(C);
        cudaStream_t fs = flux_stream(s, 1 + sub);
        if (!fs) return fail(AK_ERR_CUDA, "face-flux branch could not be forked");
        k_face_flux_fine<SF><<<dim3((unsigned)blocks3(32 * R->max_face), R->nfaces), 256, 0, fs>>>(
            src_of<SF>(F), F->G, R->d_terms[0], R->d_terms[1], R->nterms, R->d_faces, R->nfaces, R->d_offs, R->pad,
            R->dx_f * R->dx_f * R->dx_f, R->reg_f);
        if (fork && sub == 0) AK_CUDA(cudaEventRecord(R->ev_flux_f0, R->flux));
        // the walls' last block sums the loads; the second fine step's also
        // adds both steps' loads to the running sums
        if (nlinks)
            AK_CUDA(launch_chained(CHAIN_FINE, k_walls<SF>, dim3((unsigned)nb), dim3(256), s, src_of<SF>(F), F->G, F->keys,
                                   F->wall_q, F->nkeys, 1, F->n_elements, F->ox, F->oy, F->partials,
                                   R->wall_done + sub, R->d_loads + sub * 5 * F->n_elements,
                                   sub ? R->cum_loads : (double *)nullptr, (const double *)R->d_loads));
        mark(C);
        // the second fine step streams into the copy the first step's flux reads
        if (fork && sub == 1) AK_CUDA(cudaStreamWaitEvent(s, R->ev_flux_f0, 0));
        if (fine_fused && sub == 0)
            AK_CUDA(launch_chained(CHAIN_FINE, k_stream_collide<SF, false>, dim3(gfr), dim3(128), s, (const SF *)src_of<SF>(F),
                                   dst_of<SF>(F), (const uint8_t *)F->flags, F->G, F->shift_host, (TF)F->omega_s,
                                   (TF)F->omega_b, Sgs<TF>{}, make_int4(0, 0, 0, 0), fine_rect,
                                   make_int4(0, 0, 0, 0), (long long *)nullptr));
        else
            AK_CUDA(launch_chained(CHAIN_FINE, k_stream<SF>, gf, dim3(128), s, (const SF *)src_of<SF>(F), dst_of<SF>(F),
                                   (const uint8_t *)F->flags, F->G, 1));
        mark(C);
        AK_CUDA(cudaGetLastError());
        F->cur = 1 - F->cur;
        return AK_OK;
    };

    mark(C);  // step start
    // donors before the coarse step
    k_block_moments<S><<<(unsigned)split_blocks(nring_block), SPLIT_THREADS, 0, st>>>(
        src_of<S>(C), C->G, B, R->d_free, moments_of<S>(R->mom_old), nullptr, nullptr, R->d_flag);
    if (fork) {
        // the first fine step needs only the donors before the coarse step:
        // it runs on the side stream beside the coarse step (captured graphs)
        AK_CUDA(cudaEventRecord(R->ev_fork, st));
        AK_CUDA(cudaStreamWaitEvent(R->side, R->ev_fork, 0));
        AK_CUDA(cudaMemsetAsync(R->reg_f, 0, sizeof(double) * R->reg_doubles, R->side));
        AK_TRY(fine_part(0, R->side));
        AK_CUDA(cudaEventRecord(R->ev_join, R->side));
        AK_TRY(coarse_part());
        AK_CUDA(cudaStreamWaitEvent(st, R->ev_join, 0));
    } else {
        AK_TRY(coarse_part());
        AK_CUDA(cudaMemsetAsync(R->reg_f, 0, sizeof(double) * R->reg_doubles, st));
        AK_TRY(fine_part(0, st));
    }
    AK_TRY(fine_part(1, st));
    auto reflux = [&](cudaStream_t s) -> int {
        AK_CUDA(launch_chained(CHAIN_TAIL, k_reflux<S>, dim3((unsigned)split_blocks(R->max_face), R->nfaces),
                               dim3(SPLIT_THREADS), s, src_of<S>(C), C->G, (const Face *)R->d_faces, R->nfaces,
                               (const long long *)R->d_offs, (const double *)R->reg_c, (const double *)R->reg_f,
                               1.0 / (R->dx_c * R->dx_c * R->dx_c), R->d_flag));
        // the transfer block's cells outside the box are final after the
        // reflux (the restriction writes the box's): their budget sums
        if (fstats) AK_TRY(enqueue_band_sums<S>(R, s));
        return AK_OK;
    };
    if (fork) {
        // The reflux needs the face fluxes of both fine steps and the coarse
        // cells just outside the box faces, which nothing reads after the
        // donor moments that precede the second fine step: it runs on the
        // face-flux branch right after the last flux, beside the second fine
        // step's walls and streaming.  The restriction (box cells, disjoint)
        // follows the fine streaming on the step's stream, the fine block's
        // budget sums beside it.
        AK_TRY(reflux(R->flux));
        AK_CUDA(cudaEventRecord(R->ev_flux_done, R->flux));
        if (fstats) {
            AK_CUDA(cudaEventRecord(R->ev_fork, st));
            AK_CUDA(cudaStreamWaitEvent(R->side, R->ev_fork, 0));
            AK_TRY(enqueue_fine_stats<SF>(R, R->side));
            AK_CUDA(cudaEventRecord(R->ev_join, R->side));
        }
        AK_CUDA((launch_restrict<S, SF>(R, f2c, st)));
        if (fstats) AK_CUDA(cudaStreamWaitEvent(st, R->ev_join, 0));
        AK_CUDA(cudaStreamWaitEvent(st, R->ev_flux_done, 0));
    } else {
        AK_TRY(reflux(st));
        AK_CUDA((launch_restrict<S, SF>(R, f2c, st)));
    }
    AK_CUDA(cudaGetLastError());
    // leave_open: the far pass, the budget's outer flux and the reduction of
    // the coarse rows stay on their branches; the next step of the capture
    // joins them (its near pass waits for ev_far_done, its end for the rest)
    const bool open = bnd && leave_open;
    if (bnd && !open) AK_CUDA(cudaStreamWaitEvent(st, R->ev_bnd_out, 0));
    if (bnd && R->track_budget && !open) AK_CUDA(cudaStreamWaitEvent(st, R->ev_outer_out, 0));
    // a tracked budget closes on the integrals of the state the step leaves
    if (fstats) {
        if (!fork) AK_TRY(enqueue_fine_stats<SF>(R, st));
        if (open) {
            AK_CUDA(cudaEventRecord(R->ev_band_done, st));
            AK_CUDA(cudaStreamWaitEvent(R->bnd, R->ev_band_done, 0));
            AK_TRY(enqueue_coarse_rows_final(R, R->bnd));
        } else {
            AK_TRY(enqueue_coarse_rows_final(R, st));
        }
    } else if (R->track_budget && R->step_stats)
        AK_TRY((enqueue_region_stats<S, SF>(R, st)));
    if (open) AK_CUDA(cudaEventRecord(R->ev_far_done, R->bnd));
    mark(C);  // step end
    C->launches += 6 + 6 * 2 - (donors_collide ? 1 : 0) + (C->n_ubb ? 1 : 0) + (C->n_out ? 1 : 0) + (nlinks ? 0 : -2) + 1 +
                   (bnd ? 1 : 0);
    R->pre_mode = 1;
    R->pre_writes = C->pdf_writes;
    C->steps += 1;
    F->steps += 2;
    R->steps += 1;
    return AK_OK;
}

// Kernel priorities of a captured refined step: the coarse pass outside the
// transfer block (the full-lattice grid of k_stream_collide on the
// boundaries' branch) takes the device's least priority, every other kernel
// the greatest, so the short kernels of the interface chain are scheduled
// ahead of the long pass's remaining blocks as SMs free up.
template <typename S>
int graph_priorities(ak_refined *R, cudaGraph_t g) {
    ak_case *C = R->coarse;
    const unsigned far_grid = stream_collide_grid<S>(make_int4(0, 0, 0, 0), C->nx, C->ny, C->nz);
    int least = 0, greatest = 0;
    AK_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    size_t n = 0;
    AK_CUDA(cudaGraphGetNodes(g, nullptr, &n));
    std::vector<cudaGraphNode_t> nodes(n);
    AK_CUDA(cudaGraphGetNodes(g, nodes.data(), &n));
    const void *pass = (const void *)k_stream_collide<S>;
    const void *pass_stats = pass;
    if constexpr (fused_stats_form<S>()) pass_stats = (const void *)k_stream_collide<S, true>;
    for (size_t k = 0; k < n; ++k) {
        cudaGraphNodeType type;
        AK_CUDA(cudaGraphNodeGetType(nodes[k], &type));
        if (type != cudaGraphNodeTypeKernel) continue;
        cudaKernelNodeParams p{};
        AK_CUDA(cudaGraphKernelNodeGetParams(nodes[k], &p));
        cudaKernelNodeAttrValue v{};
        v.priority = (p.func == pass || p.func == pass_stats) && p.gridDim.x == far_grid ? least : greatest;
        AK_CUDA(cudaGraphKernelNodeSetAttribute(nodes[k], cudaKernelNodeAttributePriority, &v));
    }
    return AK_OK;
}

// One coarse step, or several, replayed from a CUDA graph: the steps' kernel
// sequence is captured once per buffer parity (the coarse copies swap every
// step, the fine copies twice) and the host-side counters are advanced as the
// eager step advances them.  Several steps in one graph (fused form with the
// boundaries' branch) overlap each step's first fine step, donor moments and
// transfer-block collision with the previous step's far pass.
template <typename S, typename SF>
int refined_step_graphed(ak_refined *R, int nsteps) {
    ak_case *C = R->coarse, *F = R->fine;
    const int slot = C->cur | (F->cur << 1) | (R->track_budget ? 4 : 0) | (R->step_stats ? 8 : 0) |
                     (nsteps == 4 ? 32 : (nsteps == 2 ? 16 : 0));
    if (!R->graph[slot]) {
        const int ccur = C->cur, fcur = F->cur;
        const long long cs = C->steps, fs = F->steps, rs = R->steps, cl = C->launches;
        std::vector<cudaEvent_t> *timing = C->timing;
        C->timing = nullptr;
        AK_CUDA(cudaStreamBeginCapture(C->stream, cudaStreamCaptureModeThreadLocal));
        int r = AK_OK;
        // every step but the last leaves its far pass open, every step but
        // the first waits for the previous one's
        for (int k = 0; k < nsteps && r == AK_OK; ++k)
            r = refined_step<S, SF>(R, true, k > 0, k + 1 < nsteps);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(C->stream, &g);
        C->timing = timing;
        R->graph_launches[slot] = C->launches - cl;
        C->cur = ccur;
        F->cur = fcur;
        C->steps = cs;
        F->steps = fs;
        R->steps = rs;
        C->launches = cl;
        if (r != AK_OK || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            return r != AK_OK ? r : fail(AK_ERR_CUDA, std::string("step capture failed: ") + cudaGetErrorString(e));
        }
        const bool prio = R->fused && R->bnd_branch;
        const int rp = prio ? graph_priorities<S>(R, g) : AK_OK;
        if (rp != AK_OK) {
            cudaGraphDestroy(g);
            return rp;
        }
        // the nodes' own priorities apply only with this flag
        const cudaError_t ei =
            cudaGraphInstantiate(&R->graph[slot], g, prio ? cudaGraphInstantiateFlagUseNodePriority : 0);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) {
            R->graph[slot] = nullptr;
            return fail(AK_ERR_CUDA, std::string("step graph instantiation failed: ") + cudaGetErrorString(ei));
        }
    }
    AK_CUDA(cudaGraphLaunch(R->graph[slot], C->stream));
    if (nsteps % 2) C->cur = 1 - C->cur;
    R->pre_mode = 1;
    R->pre_writes = C->pdf_writes;
    C->launches += R->graph_launches[slot];
    C->steps += nsteps;
    F->steps += 2 * nsteps;
    R->steps += nsteps;
    return AK_OK;
}

// steps replayed two per graph where the form allows it
template <typename S, typename SF>
int refined_steps_graphed(ak_refined *R, int nsteps) {
    const bool pairs = R->fused && R->bnd_branch;
    for (int s = 0; s < nsteps;) {
        const int k = !pairs ? 1 : (nsteps - s >= STEPS_PER_GRAPH ? STEPS_PER_GRAPH : (nsteps - s >= 2 ? 2 : 1));
        AK_TRY((refined_step_graphed<S, SF>(R, k)));
        s += k;
    }
    return AK_OK;
}

}  // namespace

extern "C" {

int ak_refined_create(const ak_refined_desc *desc, ak_refined **out) {
    g_error.clear();
    if (!desc || !out) return fail(AK_ERR_INVALID, "null argument");
    *out = nullptr;
    const ak_case_desc &cd = desc->coarse;
    AK_TRY(validate_desc(&cd, true));
    if (cd.farfield != AK_FARFIELD_LEGACY) return fail(AK_ERR_INVALID, "the refined solver uses the legacy outer boundary");
    if (cd.smagorinsky != 0.0) return fail(AK_ERR_INVALID, "Refined SGS is not implemented; select sgs=none explicitly");
    for (int a = 0; a < 3; ++a)
        if (desc->box_lower[a] < 0 || desc->box_upper[a] <= desc->box_lower[a])
            return fail(AK_ERR_INVALID, "fine-box bounds must have 0 <= lower < upper");
    if (desc->box_lower[2] != 0 || desc->box_upper[2] != cd.nz)
        return fail(AK_ERR_INVALID, "the fine box must span the whole periodic z axis");
    if (desc->box_lower[0] < 1 || desc->box_lower[1] < 1 || desc->box_upper[0] > cd.nx - 1 || desc->box_upper[1] > cd.ny - 1)
        return fail(AK_ERR_INVALID, "the refined box must fit strictly inside the external x/y domain");
    if (!(desc->tau_shear > 0.5) || !(desc->tau_bulk > 0.5) || !(desc->dt_coarse > 0) || !(desc->span > 0))
        return fail(AK_ERR_INVALID, "relaxation times must exceed 0.5 and dt, span be positive");
    if (desc->fine_storage >= 0 && desc->fine_storage != cd.storage &&
        !(cd.storage == AK_STORAGE_F16 && desc->fine_storage == AK_STORAGE_F32))
        return fail(AK_ERR_INVALID, "the fine level shares the coarse storage form, or holds FP32 under an FP16 "
                                    "coarse level");
    ak_refined *R = new ak_refined();
    R->dx_c = cd.dx;
    R->dt_c = desc->dt_coarse;
    R->dx_f = cd.dx / 2;
    R->dt_f = desc->dt_coarse / 2;
    R->tau_s_c = desc->tau_shear;
    R->tau_b_c = desc->tau_bulk;
    R->tau_s_f = 0.5 + 2 * (desc->tau_shear - 0.5);
    R->tau_b_f = 0.5 + 2 * (desc->tau_bulk - 0.5);
    R->span = desc->span;
    R->speed = cd.speed;
    BoxSpec &B = R->B;
    for (int a = 0; a < 3; ++a) {
        B.lo[a] = desc->box_lower[a];
        B.hi[a] = desc->box_upper[a];
    }
    B.bx = B.hi[0] - B.lo[0];
    B.by = B.hi[1] - B.lo[1];
    B.bz = B.hi[2] - B.lo[2];
    B.dx0 = B.lo[0] - 3;
    B.dy0 = B.lo[1] - 3;
    B.dnx = B.bx + 6;
    B.dny = B.by + 6;
    R->fused = B.lo[0] >= 3 && B.hi[0] + 3 <= cd.nx && B.lo[1] >= 3 && B.hi[1] + 3 <= cd.ny;
    R->xfer = make_int4(B.lo[0] - 2, B.hi[0] + 4, B.lo[1] - 2, B.hi[1] + 4);
    R->bnd_branch = B.lo[0] >= 6 && B.hi[0] + 6 <= cd.nx && B.lo[1] >= 6 && B.hi[1] + 6 <= cd.ny;
    R->near = make_int4(R->xfer.x - 1, R->xfer.y + 1, R->xfer.z - 1, R->xfer.w + 1);
    int r = AK_OK;
    // coarse lattice: no walls (they live on the fine level)
    ak_case_desc coarse = cd;
    coarse.omega_shear = 1.0 / R->tau_s_c;
    coarse.omega_bulk = 1.0 / R->tau_b_c;
    coarse.n_elements = 0;
    r = create_lattice(&coarse, AK_FARFIELD_LEGACY, false, &R->coarse);
    // fine block: two donor cells around the box in x and y, wraps everywhere
    ak_case_desc fine = cd;
    fine.storage = desc->fine_storage >= 0 ? desc->fine_storage : cd.storage;
    fine.nx = 2 * B.bx + 2 * R->pad;
    fine.ny = 2 * B.by + 2 * R->pad;
    fine.nz = 2 * B.bz;
    fine.dx = R->dx_f;
    fine.origin_x = cd.origin_x + B.lo[0] * cd.dx - R->pad * R->dx_f;
    fine.origin_y = cd.origin_y + B.lo[1] * cd.dx - R->pad * R->dx_f;
    fine.omega_shear = 1.0 / R->tau_s_f;
    fine.omega_bulk = 1.0 / R->tau_b_f;
    if (r == AK_OK) r = create_lattice(&fine, -1, true, &R->fine);
    if (r == AK_OK) {
        // every wall link must belong to the physical fine box, and the
        // donor band must be fluid
        ak_case *F = R->fine;
        std::vector<WallKey> keys((size_t)F->nkeys);
        if (F->nkeys)
            cudaMemcpy(keys.data(), F->keys, keys.size() * sizeof(WallKey), cudaMemcpyDeviceToHost);
        for (const WallKey &k : keys)
            if (k.x - 1 < R->pad + 6 || k.x - 1 >= F->nx - R->pad - 6 || k.y - 1 < R->pad + 6 ||
                k.y - 1 >= F->ny - R->pad - 6)
                r = fail(AK_ERR_INVALID, "A solid intersects the fluid donor band");
    }
    if (r == AK_OK) {
        // owned regions: coarse cells outside the fine box, the physical fine block
        const int cr[8] = {0, R->coarse->nx, 0, R->coarse->ny, B.lo[0], B.hi[0], B.lo[1], B.hi[1]};
        const int fr[8] = {R->pad, R->fine->nx - R->pad, R->pad, R->fine->ny - R->pad, 0, 0, 0, 0};
        std::copy(cr, cr + 8, R->coarse->res_region);
        std::copy(fr, fr + 8, R->fine->res_region);
        free_populations(R->speed, R->free_g);
        r = ralloc(R, &R->d_free, Q);
        if (r == AK_OK) r = cudaMemcpy(R->d_free, R->free_g, sizeof R->free_g, cudaMemcpyHostToDevice) == cudaSuccess
                                ? AK_OK : fail(AK_ERR_CUDA, "upload failed");
    }
    const long long nblock = (long long)B.dnx * B.dny * cd.nz;
    if (r == AK_OK) r = ralloc(R, &R->mom_old, (size_t)nblock * 10);
    if (r == AK_OK) r = ralloc(R, &R->mom_new, (size_t)nblock * 10);
    if (r == AK_OK) r = ralloc(R, &R->mom_half, (size_t)nblock * 10);
    if (r == AK_OK) r = ralloc(R, &R->pro_x, (size_t)(2 * B.bx + 2 * R->pad) * B.dny * cd.nz * 10);
    if (r == AK_OK) r = ralloc(R, &R->pro_x2, (size_t)(2 * B.bx + 2 * R->pad) * B.dny * cd.nz * 10);
    if (r == AK_OK) {
        R->nfaces = 0;
        long long off = 0;
        for (int axis = 0; axis < 2; ++axis)
            for (int side = -1; side <= 1; side += 2) {
                Face f{};
                f.axis = axis;
                f.side = side;
                const int b = axis == 0 ? B.bx : B.by;
                f.coarse_index = side < 0 ? B.lo[axis] - 1 : B.hi[axis] - 1;
                f.fine_index = side < 0 ? R->pad - 1 : R->pad + 2 * b - 1;
                f.lo1 = axis == 0 ? B.lo[1] : B.lo[0];
                f.n1 = axis == 0 ? B.by : B.bx;
                f.lo2 = 0;
                f.n2 = cd.nz;
                R->faces[R->nfaces] = f;
                R->offs[R->nfaces] = off;
                off += 4LL * f.n1 * f.n2;
                R->max_face = std::max<long long>(R->max_face, (long long)f.n1 * f.n2);
                ++R->nfaces;
            }
        R->reg_doubles = off;
        r = ralloc(R, &R->reg_c, (size_t)off);
        if (r == AK_OK) r = ralloc(R, &R->reg_f, (size_t)off);
        if (r == AK_OK) r = ralloc(R, &R->d_faces, 4);
        if (r == AK_OK) r = ralloc(R, &R->d_offs, 4);
        if (r == AK_OK) {
            cudaMemcpy(R->d_faces, R->faces, sizeof R->faces, cudaMemcpyHostToDevice);
            cudaMemcpy(R->d_offs, R->offs, sizeof R->offs, cudaMemcpyHostToDevice);
        }
        for (int axis = 0; axis < 2 && r == AK_OK; ++axis) {
            std::vector<FluxTerm> t = flux_terms(axis);
            R->nterms = (int)t.size();
            r = ralloc(R, &R->d_terms[axis], t.size());
            if (r == AK_OK) cudaMemcpy(R->d_terms[axis], t.data(), t.size() * sizeof(FluxTerm), cudaMemcpyHostToDevice);
        }
    }
    if (r == AK_OK) {
        // outer x and y faces of the coarse lattice, in the order x-, x+, y-, y+
        long long most = 1;
        for (int k = 0; k < 4; ++k) {
            Face f{};
            f.axis = k / 2;
            f.side = (k & 1) ? 1 : -1;
            const int n_axis = f.axis == 0 ? cd.nx : cd.ny;
            f.coarse_index = f.side < 0 ? -1 : n_axis - 1;
            f.lo1 = 0;
            f.n1 = f.axis == 0 ? cd.ny : cd.nx;
            f.lo2 = 0;
            f.n2 = cd.nz;
            R->outer[k] = f;
            most = std::max<long long>(most, (long long)f.n1 * f.n2);
        }
        R->outer_blocks = (int)blocks3(most);
        r = ralloc(R, &R->d_outer, 4);
        if (r == AK_OK) r = cudaMemcpy(R->d_outer, R->outer, sizeof R->outer, cudaMemcpyHostToDevice) == cudaSuccess
                                ? AK_OK : fail(AK_ERR_CUDA, "upload failed");
        if (r == AK_OK) r = ralloc(R, &R->outer_partials, (size_t)4 * R->outer_blocks * 4);
        const long long nl = 10LL * std::max(1, cd.n_elements);
        R->report_doubles = 1 + nl + 8 + 2 * NSTAT;
        if (r == AK_OK) r = ralloc(R, &R->report, (size_t)R->report_doubles);
        if (r == AK_OK) {
            R->d_flag = reinterpret_cast<int *>(R->report);
            R->d_loads = R->report + 1;
            R->outer_out = R->d_loads + nl;
            R->stats_out = R->outer_out + 8;
            if (cudaMallocHost((void **)&R->host_report, sizeof(double) * R->report_doubles) != cudaSuccess)
                r = fail(AK_ERR_NOMEM, "pinned host allocation failed");
        }
        if (r == AK_OK) r = ralloc(R, &R->cum_loads, (size_t)5 * std::max(1, cd.n_elements));
        if (r == AK_OK) r = ralloc(R, &R->stats_partials, (size_t)STATS_BLOCKS * NSTAT);
        // rows of the fine block's budget sums
        const long long frows = region_sum_rows(region_cells(fine_region(R), R->fine->nz));
        if (r == AK_OK) r = ralloc(R, &R->fine_rows, (size_t)frows * NSTAT);
        if (r == AK_OK) r = ralloc(R, &R->fine_stage, (size_t)blocks_for(frows, REDUCE_THREADS) * NSTAT);
        if (r == AK_OK && R->fused) {
            // rows of the fused pass's budget sums, one per warp: its far
            // launch (a grid over the whole coarse lattice), its near launch,
            // then the band's rows
            const int4 nr = R->near;
            R->cstats_far = 4 * blocks_for((long long)cd.nx * cd.ny * cd.nz, 128);
            R->cstats_near = 4 * blocks_for((long long)(nr.y - nr.x) * (nr.w - nr.z) * cd.nz, 128);
            const long long rows =
                R->cstats_far + R->cstats_near + region_sum_rows(region_cells(band_region(R), cd.nz));
            r = ralloc(R, &R->cstats, (size_t)rows * NSTAT);
            if (r == AK_OK) r = ralloc(R, &R->cstats_stage, (size_t)blocks_for(rows, REDUCE_THREADS) * NSTAT);
        }
        if (r == AK_OK && (cudaMemset(R->outer_out, 0, 8 * sizeof(double)) != cudaSuccess ||
                           cudaMemset(R->cum_loads, 0, 5 * std::max(1, cd.n_elements) * sizeof(double)) != cudaSuccess))
            r = fail(AK_ERR_CUDA, "memset failed");
    }
    if (r == AK_OK && (cudaStreamCreateWithFlags(&R->side, cudaStreamNonBlocking) != cudaSuccess ||
                       cudaStreamCreateWithFlags(&R->flux, cudaStreamNonBlocking) != cudaSuccess ||
                       cudaEventCreateWithFlags(&R->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
                       cudaEventCreateWithFlags(&R->ev_join, cudaEventDisableTiming) != cudaSuccess ||
                       cudaEventCreateWithFlags(&R->ev_flux_in[0], cudaEventDisableTiming) != cudaSuccess ||
                       cudaEventCreateWithFlags(&R->ev_flux_in[1], cudaEventDisableTiming) != cudaSuccess ||
                       cudaEventCreateWithFlags(&R->ev_flux_in[2], cudaEventDisableTiming) != cudaSuccess ||
                       cudaEventCreateWithFlags(&R->ev_flux_f0, cudaEventDisableTiming) != cudaSuccess ||
                       cudaEventCreateWithFlags(&R->ev_flux_done, cudaEventDisableTiming) != cudaSuccess ||
                       cudaStreamCreateWithFlags(&R->bnd, cudaStreamNonBlocking) != cudaSuccess ||
                       cudaEventCreateWithFlags(&R->ev_bnd_in, cudaEventDisableTiming) != cudaSuccess ||
                       cudaEventCreateWithFlags(&R->ev_bnd_out, cudaEventDisableTiming) != cudaSuccess ||
                       cudaEventCreateWithFlags(&R->ev_far_done, cudaEventDisableTiming) != cudaSuccess ||
                       cudaEventCreateWithFlags(&R->ev_band_done, cudaEventDisableTiming) != cudaSuccess ||
                       cudaStreamCreateWithFlags(&R->ostr, cudaStreamNonBlocking) != cudaSuccess ||
                       cudaEventCreateWithFlags(&R->ev_outer_in, cudaEventDisableTiming) != cudaSuccess ||
                       cudaEventCreateWithFlags(&R->ev_outer_out, cudaEventDisableTiming) != cudaSuccess))
        r = fail(AK_ERR_CUDA, "stream or event creation failed");
    if (r == AK_OK) {
        ak_case *F = R->fine;
        const long long nb = blocks_for(F->nkeys * F->nz * 3, 256);
        r = ensure_partials(F, std::max<long long>(1, nb * 5 * F->n_elements));
    }
    if (r == AK_OK) r = ralloc(R, &R->wall_done, 2);
    if (r == AK_OK) r = ralloc(R, &R->rows_done, 2);
    if (r == AK_OK && (cudaMemset(R->d_loads, 0, sizeof(double) * 2 * 5 * std::max(1, cd.n_elements)) != cudaSuccess ||
                       cudaMemset(R->wall_done, 0, 2 * sizeof(unsigned)) != cudaSuccess ||
                       cudaMemset(R->rows_done, 0, 2 * sizeof(unsigned)) != cudaSuccess))
        r = fail(AK_ERR_CUDA, "memset failed");
    if (r == AK_OK && cudaDeviceSynchronize() != cudaSuccess) r = fail(AK_ERR_CUDA, "refined set-up failed");
    if (r != AK_OK) {
        std::string keep = g_error;
        refined_release(R);
        delete R;
        g_error = keep;
        return r;
    }
    *out = R;
    return AK_OK;
}

int ak_refined_destroy(ak_refined *R) {
    if (!R) return AK_OK;
    refined_release(R);
    delete R;
    return AK_OK;
}

ak_case *ak_refined_level(ak_refined *R, int32_t level) {
    if (!R) return nullptr;
    return level == 0 ? R->coarse : (level == 1 ? R->fine : nullptr);
}

int ak_refined_init_perturbed(ak_refined *R, double amp, double phase_y, double phase_z, double lead_x,
                              double lead_y) {
    if (!R) return fail(AK_ERR_INVALID, "null case");
    return with_levels(R, [&](auto *tc, auto *tf) {
        AK_LEVEL_TYPES(tc, tf);
        return refined_init<S, SF>(R, amp, phase_y, phase_z, lead_x, lead_y);
    });
}

int ak_refined_step(ak_refined *R, int32_t nsteps, double *loads) {
    return ak_refined_step_budget(R, nsteps, loads, nullptr, nullptr);
}

int ak_refined_step_budget(ak_refined *R, int32_t nsteps, double *loads, double *outer, double *stats) {
    if (!R) return fail(AK_ERR_INVALID, "null case");
    if (nsteps < 1) return fail(AK_ERR_INVALID, "nsteps must be >= 1");
    if ((outer || stats) && !R->track_budget)
        return fail(AK_ERR_INVALID, "the outer flux and the integrals of a step need budget tracking");
    cudaStream_t st = R->coarse->stream;
    AK_CUDA(cudaMemsetAsync(R->d_flag, 0, sizeof(int), st));
    {
        // with stats every step closes its budget on the integrals of the
        // state it leaves (the reference's step, refined_solver.py:311-343);
        // the last step's are returned
        R->step_stats = stats != nullptr;
        const int r = with_levels(R, [&](auto *tc, auto *tf) {
            AK_LEVEL_TYPES(tc, tf);
            return refined_steps_graphed<S, SF>(R, nsteps);
        });
        R->step_stats = false;
        if (r != AK_OK) return r;
    }
    // flag, loads, outer flux and integrals in one copy from the report block
    AK_CUDA(cudaMemcpyAsync(R->host_report, R->report, sizeof(double) * R->report_doubles, cudaMemcpyDeviceToHost,
                            st));
    AK_CUDA(cudaStreamSynchronize(st));
    int flag = 0;
    std::memcpy(&flag, R->host_report, sizeof(int));
    const int n = R->fine->n_elements;
    const double *two = R->host_report + 1;
    if (outer) std::memcpy(outer, R->host_report + (R->outer_out - R->report), 8 * sizeof(double));
    if (stats) std::memcpy(stats, R->host_report + (R->stats_out - R->report), 2 * NSTAT * sizeof(double));
    if (flag) {
        std::string why = (flag & XF_NEGATIVE) ? "negative physical populations" :
                          (flag & XF_MACH) ? "local lattice Mach above 0.3" : "nonpositive density";
        return fail(AK_ERR_GUARD, "Refined transfer failed: " + why);
    }
    if (loads)
        for (int k = 0; k < 5 * n; ++k) loads[k] = two[k] + two[5 * n + k];
    return AK_OK;
}

int64_t ak_refined_steps_done(const ak_refined *R) { return R ? R->steps : -1; }

int ak_refined_track_budget(ak_refined *R, int32_t enable) {
    if (!R) return fail(AK_ERR_INVALID, "null case");
    R->track_budget = enable != 0;
    return AK_OK;
}

int ak_refined_outer_flux(ak_refined *R, double *out) {
    if (!R || !out) return fail(AK_ERR_INVALID, "a case and an output array are required");
    AK_CUDA(cudaStreamSynchronize(R->coarse->stream));
    AK_CUDA(cudaMemcpy(out, R->outer_out, 8 * sizeof(double), cudaMemcpyDeviceToHost));
    return AK_OK;
}

int ak_refined_restore_counters(ak_refined *R, int64_t steps, const double *cumulative_loads,
                                const double *cumulative_outer) {
    if (!R || steps < 0 || !cumulative_loads || !cumulative_outer)
        return fail(AK_ERR_INVALID, "a case, steps >= 0 and both arrays are required");
    AK_CUDA(cudaStreamSynchronize(R->coarse->stream));
    AK_CUDA(cudaMemcpy(R->cum_loads, cumulative_loads, 5 * std::max(1, R->fine->n_elements) * sizeof(double),
                       cudaMemcpyHostToDevice));
    AK_CUDA(cudaMemcpy(R->outer_out + 4, cumulative_outer, 4 * sizeof(double), cudaMemcpyHostToDevice));
    R->steps = steps;
    R->coarse->steps = steps;
    R->fine->steps = 2 * steps;
    return AK_OK;
}

int ak_refined_cumulative_loads(ak_refined *R, double *out) {
    if (!R || !out) return fail(AK_ERR_INVALID, "a case and an output array are required");
    AK_CUDA(cudaStreamSynchronize(R->coarse->stream));
    AK_CUDA(cudaMemcpy(out, R->cum_loads, 5 * std::max(1, R->fine->n_elements) * sizeof(double),
                       cudaMemcpyDeviceToHost));
    return AK_OK;
}

int ak_refined_integrals(ak_refined *R, double *out) {
    if (!R || !out) return fail(AK_ERR_INVALID, "a case and an output array are required");
    ak_case *C = R->coarse;
    cudaStream_t st = C->stream;
    const int r = with_levels(R, [&](auto *tc, auto *tf) {
        AK_LEVEL_TYPES(tc, tf);
        return enqueue_region_stats<S, SF>(R, st);
    });
    if (r != AK_OK) return r;
    AK_CUDA(cudaMemcpyAsync(out, R->stats_out, 2 * NSTAT * sizeof(double), cudaMemcpyDeviceToHost, st));
    AK_CUDA(cudaStreamSynchronize(st));
    return AK_OK;
}

int ak_refined_step_timed(ak_refined *R, int32_t nsteps, double *ms) {
    if (!R || nsteps < 1 || !ms) return fail(AK_ERR_INVALID, "a case, nsteps >= 1 and an output array are required");
    ak_case *C = R->coarse;
    std::vector<cudaEvent_t> events;
    C->timing = &events;
    int r = AK_OK;
    for (int s = 0; s < nsteps && r == AK_OK; ++s)
        r = with_levels(R, [&](auto *tc, auto *tf) {
            AK_LEVEL_TYPES(tc, tf);
            return refined_step<S, SF>(R);
        });
    C->timing = nullptr;
    const cudaError_t e = cudaStreamSynchronize(C->stream);
    for (int k = 0; k < 6; ++k) ms[k] = 0.0;
    // per step: start, cc0, cc1, cs0, cs1, (fc0, fc1, fs0, fs1) x 2, end = 14 marks
    if (r == AK_OK && e == cudaSuccess && events.size() == (size_t)14 * nsteps) {
        float t = 0.0f;
        for (int s = 0; s < nsteps; ++s) {
            cudaEvent_t *ev = events.data() + 14 * s;
            cudaEventElapsedTime(&t, ev[0], ev[13]);
            ms[0] += t;
            cudaEventElapsedTime(&t, ev[1], ev[2]);
            ms[1] += t;  // coarse collide (the transfer block alone when fused)
            cudaEventElapsedTime(&t, ev[3], ev[4]);
            ms[2] += t;  // coarse stream (fused with the next collision)
            for (int sub = 0; sub < 2; ++sub) {
                cudaEventElapsedTime(&t, ev[5 + 4 * sub], ev[6 + 4 * sub]);
                ms[3] += t;  // fine collide
                cudaEventElapsedTime(&t, ev[7 + 4 * sub], ev[8 + 4 * sub]);
                ms[4] += t;  // fine stream
            }
        }
        ms[5] = ms[0] - ms[1] - ms[2] - ms[3] - ms[4];  // transfers, fluxes, boundaries, walls
    }
    for (cudaEvent_t ev : events) cudaEventDestroy(ev);
    if (r != AK_OK) return r;
    AK_CUDA(e);
    return AK_OK;
}

int ak_refined_states(ak_refined *R, double *coarse, double *fine) {
    if (!R) return fail(AK_ERR_INVALID, "null case");
    ak_case *C = R->coarse;
    if (coarse && R->fused) {
        if (R->pre_mode < 0 || C->pdf_writes != R->pre_writes)
            return fail(AK_ERR_INVALID, "the pre-collision coarse state is known again after the next step (the "
                                        "coarse populations were written from outside the step)");
        const long long n = (long long)C->nx * C->ny * C->nz;
        AK_TRY(ensure_staging(C, (size_t)n * Q));
        AK_TRY(with_storage(C, [&](auto *tag) {
            using S = std::remove_pointer_t<decltype(tag)>;
            k_export_pre_collision<S><<<(unsigned)blocks_for(n, 256), 256, 0, C->stream>>>(
                src_of<S>(C), dst_of<S>(C), C->G, R->xfer, R->pre_mode, C->staging);
            AK_CUDA(cudaGetLastError());
            return AK_OK;
        }));
        AK_CUDA(cudaMemcpyAsync(coarse, C->staging, n * Q * sizeof(double), cudaMemcpyDeviceToHost, C->stream));
        AK_CUDA(cudaStreamSynchronize(C->stream));
    } else if (coarse) {
        AK_TRY(ak_get_pdf(C, coarse));
    }
    if (fine) AK_TRY(ak_get_pdf(R->fine, fine));
    return AK_OK;
}

int ak_refined_probe(ak_refined *R, int32_t op, double *out, int64_t *n_out) {
    if (!R || op < 0 || op > 3) return fail(AK_ERR_INVALID, "a case and an operation 0..3 are required");
    if (n_out) *n_out = op == 2 ? 2 * R->reg_doubles : 0;
    if (op == 2 && !out) return AK_OK;
    ak_case *C = R->coarse, *F = R->fine;
    cudaStream_t st = C->stream;
    const BoxSpec &B = R->B;
    AK_CUDA(cudaStreamSynchronize(st));
    AK_CUDA(cudaMemsetAsync(R->d_flag, 0, sizeof(int), st));
    const int r = with_levels(R, [&](auto *tc, auto *tf) -> int {
        AK_LEVEL_TYPES(tc, tf);
        if (op == 0) {
            const long long nring_block = ring_count(B.dnx, B.dny, DONOR_RING, DONOR_RING) * C->nz;
            const long long nprox = ring_count(F->nx, B.dny, R->pad, DONOR_RING) * C->nz;
            const long long nband = ring_count(F->nx, F->ny, R->pad, R->pad) * F->nz;
            const Rescale c2f{R->tau_s_f * R->dt_f / (R->tau_s_c * R->dt_c),
                              R->tau_b_f * R->dt_f / (R->tau_b_c * R->dt_c)};
            k_block_moments<S><<<(unsigned)split_blocks(nring_block), SPLIT_THREADS, 0, st>>>(
                src_of<S>(C), C->G, B, R->d_free, moments_of<S>(R->mom_old), nullptr, nullptr, R->d_flag);
            k_prolong_x<<<(unsigned)blocks3(nprox), 256, 0, st>>>(B, C->nz, R->pad, moments_of<S>(R->mom_old),
                                                                   moments_of<S>(R->pro_x));
            k_donors<SF><<<(unsigned)split_blocks(nband), SPLIT_THREADS, 0, st>>>(src_of<SF>(F), F->G, C->nz,
                                                                                  moments_of<S>(R->pro_x), B.dny, c2f, R->pad,
                                                                                  R->d_flag);
        } else if (op == 1) {
            const Rescale f2c{R->tau_s_c * R->dt_c / (R->tau_s_f * R->dt_f),
                              R->tau_b_c * R->dt_c / (R->tau_b_f * R->dt_f)};
            AK_CUDA((launch_restrict<S, SF>(R, f2c, st)));
        } else if (op == 2) {
            AK_CUDA(cudaMemsetAsync(R->reg_f, 0, sizeof(double) * R->reg_doubles, st));
            k_face_flux_coarse<S><<<dim3((unsigned)blocks3(32 * R->max_face), R->nfaces), 256, 0, st>>>(
                src_of<S>(C), C->G, R->d_terms[0], R->d_terms[1], R->nterms, R->d_faces, R->nfaces, R->d_offs,
                R->dx_c * R->dx_c * R->dx_c, R->reg_c);
            k_face_flux_fine<SF><<<dim3((unsigned)blocks3(32 * R->max_face), R->nfaces), 256, 0, st>>>(
                src_of<SF>(F), F->G, R->d_terms[0], R->d_terms[1], R->nterms, R->d_faces, R->nfaces, R->d_offs,
                R->pad, R->dx_f * R->dx_f * R->dx_f, R->reg_f);
        } else {
            k_reflux<S><<<dim3((unsigned)split_blocks(R->max_face), R->nfaces), SPLIT_THREADS, 0, st>>>(
                src_of<S>(C), C->G, R->d_faces, R->nfaces, R->d_offs, R->reg_c, R->reg_f,
                1.0 / (R->dx_c * R->dx_c * R->dx_c), R->d_flag);
        }
        AK_CUDA(cudaGetLastError());
        return AK_OK;
    });
    if (r != AK_OK) return r;
    if (op == 2) {
        AK_CUDA(cudaMemcpyAsync(out, R->reg_c, sizeof(double) * R->reg_doubles, cudaMemcpyDeviceToHost, st));
        AK_CUDA(cudaMemcpyAsync(out + R->reg_doubles, R->reg_f, sizeof(double) * R->reg_doubles,
                                cudaMemcpyDeviceToHost, st));
    }
    int flag = 0;
    AK_CUDA(cudaMemcpyAsync(&flag, R->d_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    AK_CUDA(cudaStreamSynchronize(st));
    if (flag) return fail(AK_ERR_NONFINITE, "a transfer check failed (flag " + std::to_string(flag) + ")");
    return AK_OK;
}

}  // extern "C"

// ==================================================================== batch
// Independent uniform cases with the characteristic farfield, stepped by one
// set of launches per step (ak_batch.cuh).  The batch borrows the cases: it
// owns only its descriptors, work tables, stream and graphs.
struct ak_batch {
    std::vector<ak_case *> cases;
    std::vector<int> cur0;
    int storage = 0, device = 0, sms = 0;
    cudaStream_t stream = nullptr;
    void *d_cases = nullptr;
    WorkItem *w_ring = nullptr, *w_ff = nullptr, *w_walls = nullptr, *w_bulk = nullptr, *w_ubb = nullptr,
             *w_out = nullptr;
    long long n_ring = 0, n_ff = 0, n_walls = 0, n_bulk = 0, n_ubb = 0, n_out = 0;
    double *loads = nullptr;  // [case][MAX_ELEMENTS * 5]
    int parity = 0;
    long long steps = 0, launches = 0;
    // stream-collide schedule: block width, CTAs per SM of the persistent
    // grid, table order (0 case-major, 1 interleaved)
    int tb = 128, per_sm = 4, order = 0;
    cudaGraphExec_t graph[4] = {};  // (parity, sample)
    // inside the graphs the walls run on a side stream beside the farfield
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
};

namespace {

void batch_drop_graphs(ak_batch *B) {
    for (cudaGraphExec_t &g : B->graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
}

void batch_release(ak_batch *B) {
    if (B->stream) cudaStreamSynchronize(B->stream);
    batch_drop_graphs(B);
    for (void *p : {(void *)B->d_cases, (void *)B->w_ring, (void *)B->w_ff, (void *)B->w_walls, (void *)B->w_bulk,
                    (void *)B->w_ubb, (void *)B->w_out, (void *)B->loads})
        if (p) cudaFree(p);
    if (B->ev_fork) cudaEventDestroy(B->ev_fork);
    if (B->ev_join) cudaEventDestroy(B->ev_join);
    if (B->side) cudaStreamDestroy(B->side);
    if (B->stream) cudaStreamDestroy(B->stream);
}

int upload_work(WorkItem **dst, const std::vector<WorkItem> &v) {
    if (*dst) cudaFree(*dst);
    *dst = nullptr;
    const size_t n = std::max<size_t>(1, v.size());
    cudaError_t e = cudaMalloc((void **)dst, n * sizeof(WorkItem));
    if (e != cudaSuccess)
        return fail(e == cudaErrorMemoryAllocation ? AK_ERR_NOMEM : AK_ERR_CUDA,
                    std::string("batch table allocation failed: ") + cudaGetErrorString(e));
    if (!v.empty()) AK_CUDA(cudaMemcpy(*dst, v.data(), v.size() * sizeof(WorkItem), cudaMemcpyHostToDevice));
    return AK_OK;
}

// chunks of 256 items per case, case after case
std::vector<WorkItem> chunk_table(const std::vector<long long> &items) {
    std::vector<WorkItem> out;
    for (size_t c = 0; c < items.size(); ++c)
        for (long long k = 0; k < blocks_for(items[c], 256); ++k) out.push_back(WorkItem{(int)c, (int)k});
    return out;
}

// the stream-collide blocks of every case for block width tb
std::vector<WorkItem> bulk_table(const ak_batch *B, int tb, int order) {
    std::vector<long long> count;
    // the single-case kernel's items (cells, or cell pairs in the pair forms)
    for (const ak_case *c : B->cases) {
        const bool pair = c->storage == AK_STORAGE_F32 || c->storage == AK_STORAGE_F16;
        const long long items = pair ? stream_collide_items<float>(make_int4(0, 0, 0, 0), c->nx, c->ny, c->nz)
                                     : stream_collide_items<double>(make_int4(0, 0, 0, 0), c->nx, c->ny, c->nz);
        count.push_back(blocks_for(items, tb));
    }
    std::vector<WorkItem> out;
    if (order == 0) {
        for (size_t c = 0; c < count.size(); ++c)
            for (long long k = 0; k < count[c]; ++k) out.push_back(WorkItem{(int)c, (int)k});
    } else {
        // round robin over the cases, so every stretch of the table mixes cases
        const long long most = *std::max_element(count.begin(), count.end());
        for (long long k = 0; k < most; ++k)
            for (size_t c = 0; c < count.size(); ++c)
                if (k < count[c]) out.push_back(WorkItem{(int)c, (int)k});
    }
    return out;
}

// grid: the persistent grid of the looping forms; the pair forms launch one
// block per table entry
template <typename S>
int bulk_launch(ak_batch *B, int tb, int grid, int parity) {
    const BatchCase<S> *cases = (const BatchCase<S> *)B->d_cases;
    if constexpr (pair_form<S>()) grid = (int)std::max<long long>(1, B->n_bulk);
    switch (tb) {
    case 64: k_batch_bulk<S, 64><<<grid, 64, 0, B->stream>>>(cases, B->w_bulk, B->n_bulk, parity); break;
    case 128: k_batch_bulk<S, 128><<<grid, 128, 0, B->stream>>>(cases, B->w_bulk, B->n_bulk, parity); break;
    case 256: k_batch_bulk<S, 256><<<grid, 256, 0, B->stream>>>(cases, B->w_bulk, B->n_bulk, parity); break;
    default: return fail(AK_ERR_INVALID, "unsupported block width");
    }
    AK_CUDA(cudaGetLastError());
    return AK_OK;
}

template <typename S>
int bulk_occupancy(int tb, int *blocks) {
    cudaError_t e = cudaErrorInvalidValue;
    if (tb == 64) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_batch_bulk<S, 64>, 64, 0);
    if (tb == 128) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_batch_bulk<S, 128>, 128, 0);
    if (tb == 256) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_batch_bulk<S, 256>, 256, 0);
    if (e != cudaSuccess) return fail(AK_ERR_CUDA, std::string("occupancy query failed: ") + cudaGetErrorString(e));
    return AK_OK;
}

// branch: the walls (and their load sums) on the side stream, forked before
// the farfield and joined before the stream-collide; they touch disjoint
// cells (solid cells against ghost cells), as in the single-case step
template <typename S>
int batch_enqueue(ak_batch *B, int parity, bool sample, bool branch = false) {
    const BatchCase<S> *cases = (const BatchCase<S> *)B->d_cases;
    cudaStream_t ws = B->stream;
    if (branch) {
        AK_CUDA(cudaEventRecord(B->ev_fork, B->stream));
        AK_CUDA(cudaStreamWaitEvent(B->side, B->ev_fork, 0));
        ws = B->side;
    }
    if (B->n_ring) {
        k_batch_ring_macros<S><<<(unsigned)B->n_ring, 256, 0, B->stream>>>(cases, B->w_ring, parity);
        AK_CUDA(cudaGetLastError());
    }
    if (B->n_ff) {
        k_batch_farfield<S><<<(unsigned)B->n_ff, 256, 0, B->stream>>>(cases, B->w_ff, parity);
        AK_CUDA(cudaGetLastError());
    }
    if (B->n_ubb) {
        k_batch_ubb<S><<<(unsigned)B->n_ubb, 256, 0, B->stream>>>(cases, B->w_ubb, parity);
        AK_CUDA(cudaGetLastError());
    }
    if (B->n_out) {
        k_batch_outflow<S><<<(unsigned)B->n_out, 256, 0, B->stream>>>(cases, B->w_out, parity);
        AK_CUDA(cudaGetLastError());
    }
    if (B->n_walls) {
        k_batch_walls<S><<<(unsigned)B->n_walls, 256, 0, ws>>>(cases, B->w_walls, parity, sample ? 1 : 0);
        AK_CUDA(cudaGetLastError());
    }
    if (sample) {
        k_batch_sum_partials<S><<<dim3(5 * MAX_ELEMENTS, (unsigned)B->cases.size()), 32, 0, ws>>>(cases,
                                                                                              B->loads);
        AK_CUDA(cudaGetLastError());
    }
    if (branch) {
        AK_CUDA(cudaEventRecord(B->ev_join, B->side));
        AK_CUDA(cudaStreamWaitEvent(B->stream, B->ev_join, 0));
    }
    AK_TRY(bulk_launch<S>(B, B->tb, B->per_sm * B->sms, parity));
    return AK_OK;
}

long long batch_step_launches(const ak_batch *B, bool sample) {
    return (B->n_ring ? 1 : 0) + (B->n_ff ? 1 : 0) + (B->n_ubb ? 1 : 0) + (B->n_out ? 1 : 0) + (B->n_walls ? 1 : 0) +
           (sample ? 1 : 0) + 1;
}

template <typename S>
int batch_build(ak_batch *B) {
    std::vector<BatchCase<S>> host;
    std::vector<long long> ring, ff, walls, ubb, outflow;
    for (size_t i = 0; i < B->cases.size(); ++i) {
        ak_case *c = B->cases[i];
        BatchCase<S> d{};
        d.pdf[0] = (S *)c->pdf[0];
        d.pdf[1] = (S *)c->pdf[1];
        d.flags = c->flags;
        d.G = c->G;
        d.omega_s = (typename Store<S>::T)c->omega_s;
        d.sgs = sgs_of<S>(c);
        d.omega_b = (typename Store<S>::T)c->omega_b;
        d.cur0 = B->cur0[i];
        d.n_elements = c->n_elements;
        d.ox = c->ox;
        d.oy = c->oy;
        d.ubb_cells = c->ubb_cells;
        d.n_ubb_cells = c->n_ubb_cells;
        d.speed = c->speed;
        d.sel_out = c->sel_out;
        d.n_out = c->n_out;
        d.out_state = c->out_state;
        d.L = c->outer();
        d.P = c->ff();
        d.R = c->ring();
        d.ff_in = c->ff_in;
        d.ff_der = c->ff_der;
        d.ff_clock = c->ff_clock;
        d.ff_lo = c->ff_lo;
        d.ff_hi = c->ff_hi;
        d.keys = c->keys;
        d.wall_q = c->wall_q;
        d.nkeys = c->nkeys;
        const long long nlinks = c->nkeys * c->nz * 3;
        d.wall_blocks = blocks_for(nlinks, 256);
        if (nlinks) AK_TRY(ensure_partials(c, d.wall_blocks * 5 * c->n_elements));
        d.partials = c->partials;
        host.push_back(d);
        const bool legacy = c->farfield == AK_FARFIELD_LEGACY;
        ring.push_back(legacy ? 0 : c->ring_n * c->nz);
        ff.push_back(legacy ? 0 : c->nouter);
        ubb.push_back(legacy ? c->n_ubb_cells * c->nz : 0);
        outflow.push_back(legacy ? c->n_out : 0);
        walls.push_back(nlinks);
    }
    AK_CUDA(cudaMalloc(&B->d_cases, host.size() * sizeof(BatchCase<S>)));
    AK_CUDA(cudaMemcpy(B->d_cases, host.data(), host.size() * sizeof(BatchCase<S>), cudaMemcpyHostToDevice));
    const std::vector<WorkItem> tr = chunk_table(ring), tf = chunk_table(ff), tw = chunk_table(walls),
                                tu = chunk_table(ubb), to = chunk_table(outflow);
    B->n_ring = (long long)tr.size();
    B->n_ff = (long long)tf.size();
    B->n_walls = (long long)tw.size();
    B->n_ubb = (long long)tu.size();
    B->n_out = (long long)to.size();
    AK_TRY(upload_work(&B->w_ring, tr));
    AK_TRY(upload_work(&B->w_ff, tf));
    AK_TRY(upload_work(&B->w_walls, tw));
    AK_TRY(upload_work(&B->w_ubb, tu));
    AK_TRY(upload_work(&B->w_out, to));
    const std::vector<WorkItem> tb = bulk_table(B, B->tb, B->order);
    B->n_bulk = (long long)tb.size();
    AK_TRY(upload_work(&B->w_bulk, tb));
    int occ = 0;
    AK_TRY(bulk_occupancy<S>(B->tb, &occ));
    B->per_sm = std::max(1, occ);
    AK_CUDA(cudaMalloc(&B->loads, B->cases.size() * 5 * MAX_ELEMENTS * sizeof(double)));
    AK_CUDA(cudaMemset(B->loads, 0, B->cases.size() * 5 * MAX_ELEMENTS * sizeof(double)));
    return AK_OK;
}

// one batch step from a CUDA graph captured per (parity, sample)
template <typename S>
int batch_step_graphed(ak_batch *B, bool sample) {
    const int slot = B->parity | (sample ? 2 : 0);
    if (!B->side) {
        if (cudaStreamCreateWithFlags(&B->side, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&B->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&B->ev_join, cudaEventDisableTiming) != cudaSuccess)
            return fail(AK_ERR_CUDA, "stream or event creation failed");
    }
    if (!B->graph[slot]) {
        AK_CUDA(cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal));
        const int r = batch_enqueue<S>(B, B->parity, sample, true);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(B->stream, &g);
        if (r != AK_OK || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            return r != AK_OK ? r : fail(AK_ERR_CUDA, std::string("batch capture failed: ") + cudaGetErrorString(e));
        }
        const cudaError_t ei = cudaGraphInstantiate(&B->graph[slot], g, 0);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) {
            B->graph[slot] = nullptr;
            return fail(AK_ERR_CUDA, std::string("batch graph instantiation failed: ") + cudaGetErrorString(ei));
        }
    }
    AK_CUDA(cudaGraphLaunch(B->graph[slot], B->stream));
    B->launches += batch_step_launches(B, sample);
    B->parity ^= 1;
    B->steps += 1;
    return AK_OK;
}

template <typename F>
int batch_dispatch(ak_batch *B, F &&f) {
    switch (B->storage) {
    case AK_STORAGE_F64: return f((double *)nullptr);
    case AK_STORAGE_F32: return f((float *)nullptr);
    case AK_STORAGE_F16: return f((__half *)nullptr);
    case AK_STORAGE_DF64: return f((df2 *)nullptr);
    }
    return fail(AK_ERR_INVALID, "unknown storage");
}

// the cases' host-side state after the batch's steps
void batch_sync_cases(ak_batch *B, long long nsteps) {
    for (size_t i = 0; i < B->cases.size(); ++i) {
        ak_case *c = B->cases[i];
        c->cur = B->cur0[i] ^ B->parity;
        c->steps += nsteps;
    }
}

}  // namespace

extern "C" {

int ak_batch_create(ak_case *const *cases, int32_t n, ak_batch **out) {
    if (!out) return fail(AK_ERR_INVALID, "an output handle is required");
    *out = nullptr;
    if (!cases || n < 1) return fail(AK_ERR_INVALID, "a batch needs at least one case");
    ak_batch *B = new ak_batch();
    int r = AK_OK;
    for (int i = 0; i < n && r == AK_OK; ++i) {
        ak_case *c = cases[i];
        if (!c)
            r = fail(AK_ERR_INVALID, "null case in the batch");
        else if (i && (c->storage != cases[0]->storage || c->device != cases[0]->device))
            r = fail(AK_ERR_INVALID, "the cases of a batch share one storage form and one device");
        else if ((c->farfield != AK_FARFIELD_CHARACTERISTIC && c->farfield != AK_FARFIELD_LEGACY) || c->periodic_xy)
            r = fail(AK_ERR_INVALID, "batches hold uniform cases with the characteristic or the legacy outer boundary");
        else if (std::find(B->cases.begin(), B->cases.end(), c) != B->cases.end())
            r = fail(AK_ERR_INVALID, "a case appears twice in the batch");
        else
            B->cases.push_back(c);
    }
    if (r == AK_OK) {
        ak_case *c0 = B->cases[0];
        B->storage = c0->storage;
        B->device = c0->device;
        if (cudaSetDevice(B->device) != cudaSuccess ||
            cudaDeviceGetAttribute(&B->sms, cudaDevAttrMultiProcessorCount, B->device) != cudaSuccess)
            r = fail(AK_ERR_CUDA, "device query failed");
    }
    if (r == AK_OK && cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking) != cudaSuccess)
        r = fail(AK_ERR_CUDA, "stream creation failed");
    // boundary data of cases that have not stepped yet, then hand-over
    for (size_t i = 0; r == AK_OK && i < B->cases.size(); ++i) {
        ak_case *c = B->cases[i];
        if (!c->prepared)
            r = with_storage(c, [&](auto *tag) {
                using S = std::remove_pointer_t<decltype(tag)>;
                if (c->farfield != AK_FARFIELD_LEGACY) return prepare_boundaries<S>(c);
                // a legacy case that has not stepped: its outflow history is
                // seeded as the first step seeds it, after the UBB (which the
                // batch's first step applies again to the same state, writing
                // the same values)
                const int TB = 256;
                if (c->n_ubb)
                    k_ubb<S><<<(unsigned)blocks_for(c->n_ubb_cells * c->nz, TB), TB, 0, c->stream>>>(
                        src_of<S>(c), c->G, c->ubb_cells, c->n_ubb_cells, c->speed, 0.0, 0.0);
                if (c->n_out)
                    k_outflow_prepare<S><<<(unsigned)blocks_for(c->n_out, TB), TB, 0, c->stream>>>(
                        src_of<S>(c), c->G, c->outer(), c->sel_out, c->n_out, c->out_state, 1, 0, 0, 1.0, c->speed,
                        0.0, 0.0);
                AK_CUDA(cudaGetLastError());
                c->prepared = true;
                return AK_OK;
            });
        if (r == AK_OK && cudaStreamSynchronize(c->stream) != cudaSuccess) r = fail(AK_ERR_CUDA, "case sync failed");
        B->cur0.push_back(c->cur);
    }
    if (r == AK_OK) r = batch_dispatch(B, [&](auto *tag) { return batch_build<std::remove_pointer_t<decltype(tag)>>(B); });
    if (r != AK_OK) {
        std::string keep = g_error;
        batch_release(B);
        delete B;
        g_error = keep;
        return r;
    }
    *out = B;
    return AK_OK;
}

int ak_batch_destroy(ak_batch *B) {
    if (!B) return AK_OK;
    batch_release(B);
    delete B;
    return AK_OK;
}

int ak_batch_step(ak_batch *B, int32_t nsteps, double *loads) {
    if (!B) return fail(AK_ERR_INVALID, "null batch");
    if (nsteps < 1) return fail(AK_ERR_INVALID, "nsteps must be >= 1");
    for (size_t i = 0; i < B->cases.size(); ++i)
        if (B->cases[i]->cur != (B->cur0[i] ^ B->parity))
            return fail(AK_ERR_INVALID, "a case of the batch was stepped outside it; rebuild the batch");
    AK_CUDA(cudaSetDevice(B->device));
    int r = AK_OK;
    long long done = 0;
    for (int s = 0; s < nsteps && r == AK_OK; ++s) {
        const bool sample = loads && s == nsteps - 1;
        r = batch_dispatch(B, [&](auto *tag) {
            return batch_step_graphed<std::remove_pointer_t<decltype(tag)>>(B, sample);
        });
        if (r == AK_OK) ++done;
    }
    batch_sync_cases(B, done);
    if (r != AK_OK) return r;
    if (loads)
        AK_CUDA(cudaMemcpyAsync(loads, B->loads, B->cases.size() * 5 * MAX_ELEMENTS * sizeof(double),
                                cudaMemcpyDeviceToHost, B->stream));
    AK_CUDA(cudaStreamSynchronize(B->stream));
    return AK_OK;
}

int ak_batch_tune(ak_batch *B, int32_t trials, double *report) {
    if (!B || trials < 1) return fail(AK_ERR_INVALID, "a batch and trials >= 1 are required");
    AK_CUDA(cudaSetDevice(B->device));
    // the stream-collide launch reads one copy and writes the other's fluid
    // cells, which the next step rewrites whole: timing it leaves no trace
    return batch_dispatch(B, [&](auto *tag) -> int {
        using S = std::remove_pointer_t<decltype(tag)>;
        cudaEvent_t a, b;
        AK_CUDA(cudaEventCreate(&a));
        AK_CUDA(cudaEventCreate(&b));
        const int tb0 = B->tb, per0 = B->per_sm, order0 = B->order;
        double best = 1e30, first = 0.0;
        int best_tb = tb0, best_per = per0, best_order = order0;
        int r = AK_OK;
        for (int order = 0; order < 2 && r == AK_OK; ++order)
            for (int tb : {64, 128, 256}) {
                if (r != AK_OK) break;
                int occ = 0;
                r = bulk_occupancy<S>(tb, &occ);
                if (r != AK_OK || occ < 1) break;
                const std::vector<WorkItem> t = bulk_table(B, tb, order);
                B->n_bulk = (long long)t.size();
                r = upload_work(&B->w_bulk, t);
                // the pair forms' grid is their table: one timing per width and order
                for (int per = pair_form<S>() ? occ : 1; per <= occ && r == AK_OK; per *= 2) {
                    r = bulk_launch<S>(B, tb, per * B->sms, B->parity);  // warm
                    cudaEventRecord(a, B->stream);
                    for (int k = 0; k < trials && r == AK_OK; ++k) r = bulk_launch<S>(B, tb, per * B->sms, B->parity);
                    cudaEventRecord(b, B->stream);
                    if (cudaEventSynchronize(b) != cudaSuccess) r = fail(AK_ERR_CUDA, "tuning launch failed");
                    float ms = 0.0f;
                    cudaEventElapsedTime(&ms, a, b);
                    const double per_launch = ms / trials;
                    if (tb == tb0 && order == order0 && per == per0) first = per_launch;
                    if (r == AK_OK && per_launch < best) {
                        best = per_launch;
                        best_tb = tb;
                        best_per = per;
                        best_order = order;
                    }
                    B->launches += trials + 1;
                }
            }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        if (r != AK_OK) return r;
        B->tb = best_tb;
        B->per_sm = best_per;
        B->order = best_order;
        const std::vector<WorkItem> t = bulk_table(B, B->tb, B->order);
        B->n_bulk = (long long)t.size();
        AK_TRY(upload_work(&B->w_bulk, t));
        batch_drop_graphs(B);
        if (report) {
            report[0] = B->tb;
            report[1] = B->per_sm;
            report[2] = B->order;
            report[3] = best;
            report[4] = first;
        }
        return AK_OK;
    });
}

int64_t ak_batch_launches(const ak_batch *B) { return B ? B->launches : -1; }
int64_t ak_batch_steps_done(const ak_batch *B) { return B ? B->steps : -1; }
void *ak_batch_stream(const ak_batch *B) { return B ? (void *)B->stream : nullptr; }

}  // extern "C"
