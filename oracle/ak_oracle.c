/*
 * ak_oracle.c -- CPU restatement of AeroKinetic's D3Q27 cumulant time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA engine in
 * aerokinetic_gb300/csrc is compared against.  It is loaded by tests/, by
 * __graft_entry__.smoke() and by the cpu_baseline leg of bench.py, and by
 * nothing in the product.
 *
 * The reference (Bulbulator72/Aerokinetic 0.5.3) generates its per-cell code at
 * run time with lbmpy 1.4 / pystencils 1.4 (pyproject.toml:12), which is not
 * vendored.  What follows restates the published algorithms that the
 * reference configures, at the reference's own call sites:
 *
 *   - cumulant collision, Geier et al. 2015 (doi:10.1016/j.camwa.2015.05.001),
 *     compressible, zero-centred storage g_i = f_i - w_i, shear rate omega on
 *     the five deviatoric second-order cumulants, bulk rate on the trace, and
 *     rate 1 on every cumulant of order >= 3 (solver.py:75-77,
 *     interface.py:124-128; lbmpy assigns 1 to all non-shear moments when one
 *     rate is given);
 *   - pull streaming "stream_collide" into a second array (solver.py:82-85,
 *     step at solver.py:257-261), one ghost layer, periodic ghost copy;
 *   - NoSlipLinearBouzidi (Bouzidi, Firdaouss, Lallemand 2001) with the q<0
 *     half-way fallback (solver.py:100-143);
 *   - compressible UBB (solver.py:131) and ExtrapolationOutflow after Geier
 *     et al. 2015 appendix F (solver.py:133-135);
 *   - the characteristic farfield of farfield.py:144-206;
 *   - momentum-exchange loads of solver.py:204-250;
 *   - the Smagorinsky shear rate of sgs="smagorinsky" (solver.py:74-77).
 *
 * Layout: every population array is (NX, NY, NZ, 27) C-order doubles with one
 * ghost layer, NX = nx+2 etc., exactly the reference's pdf[x, y, z, d] view
 * with ghost_layers=1.  Directions follow lbmpy's D3Q27 order.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define Q 27

static const int CV[Q][3] = {
    {0, 0, 0},   {0, 1, 0},   {0, -1, 0},  {-1, 0, 0},  {1, 0, 0},   {0, 0, 1},
    {0, 0, -1},  {-1, 1, 0},  {1, 1, 0},   {-1, -1, 0}, {1, -1, 0},  {0, 1, 1},
    {0, -1, 1},  {-1, 0, 1},  {1, 0, 1},   {0, 1, -1},  {0, -1, -1}, {-1, 0, -1},
    {1, 0, -1},  {1, 1, 1},   {-1, 1, 1},  {1, -1, 1},  {-1, -1, 1}, {1, 1, -1},
    {-1, 1, -1}, {1, -1, -1}, {-1, -1, -1}};

static double W[Q];
static int INV[Q];
static int LINE[3][3][3]; /* (cx+1, cy+1, cz+1) -> direction index */

static int initialised = 0;

static void init_tables(void) {
    if (initialised) return;
    for (int q = 0; q < Q; ++q) {
        int nz = 0;
        double w = 1.0;
        for (int a = 0; a < 3; ++a) {
            w *= CV[q][a] == 0 ? 2.0 / 3.0 : 1.0 / 6.0;
            nz += CV[q][a] != 0;
        }
        (void)nz;
        W[q] = w;
        LINE[CV[q][0] + 1][CV[q][1] + 1][CV[q][2] + 1] = q;
    }
    for (int q = 0; q < Q; ++q)
        for (int p = 0; p < Q; ++p)
            if (CV[p][0] == -CV[q][0] && CV[p][1] == -CV[q][1] && CV[p][2] == -CV[q][2]) INV[q] = p;
    initialised = 1;
}

void ako_stencil(int *c, double *w, int *inv) {
    init_tables();
    for (int q = 0; q < Q; ++q) {
        for (int a = 0; a < 3; ++a) c[3 * q + a] = CV[q][a];
        w[q] = W[q];
        inv[q] = INV[q];
    }
}

/* ---- one-dimensional three-point moment transforms (Geier 2015, sec. 4) ---- */
static inline void forward_line(double *m, double u) {
    double fm = m[0], f0 = m[1], fp = m[2];
    double m0 = fm + f0 + fp;
    double d = fp - fm;
    m[0] = m0;
    m[1] = d - u * m0;
    m[2] = (fp + fm) - 2.0 * u * d + u * u * m0;
}

static inline void backward_line(double *m, double u) {
    double m0 = m[0], m1 = m[1], m2 = m[2];
    m[1] = m0 * (1.0 - u * u) - 2.0 * u * m1 - m2;
    m[2] = 0.5 * (m0 * (u * u + u) + m1 * (2.0 * u + 1.0) + m2);
    m[0] = 0.5 * (m0 * (u * u - u) + m1 * (2.0 * u - 1.0) + m2);
}

/* Smagorinsky shear rate of one cell (solver.py:74-77 selects lbmpy's
 * SMAGORINSKY subgrid model for sgs="smagorinsky"; the model is Hou, Sterling,
 * Chen & Doolen 1996 in its lattice form): with the non-equilibrium second
 * moments Pi_ab = K_ab - rho/3 delta_ab (K the central moments) and
 * |Pi| = sqrt(2 Pi:Pi) / rho, the effective relaxation time is
 * tau = (tau0 + sqrt(tau0^2 + 18 C^2 |Pi|)) / 2 with tau0 = 1/omega, the
 * molecular value.  c18 = 18 C^2; 0 keeps the molecular rate. */
static double smagorinsky_rate(double omega, double c18, double rho, double pxx, double pyy, double pzz,
                               double pxy, double pxz, double pyz) {
    const double tau0 = 1.0 / omega;
    const double norm = sqrt(2.0 * (pxx * pxx + pyy * pyy + pzz * pzz + 2.0 * (pxy * pxy + pxz * pxz + pyz * pyz))) /
                        rho;
    return 2.0 / (tau0 + sqrt(c18 * norm + tau0 * tau0));
}

/* Cumulant collision of one cell, in place on zero-centred populations g;
 * c18 > 0 replaces omega_s by the cell's Smagorinsky rate. */
static void collide_cell_sgs(double *g, double omega_s, double omega_b, double c18) {
    double K[3][3][3];
    double drho = 0.0, j[3] = {0.0, 0.0, 0.0};
    for (int q = 0; q < Q; ++q) {
        drho += g[q];
        for (int a = 0; a < 3; ++a) j[a] += CV[q][a] * g[q];
    }
    double rho = 1.0 + drho;
    double u[3] = {j[0] / rho, j[1] / rho, j[2] / rho};
    for (int q = 0; q < Q; ++q) K[CV[q][0] + 1][CV[q][1] + 1][CV[q][2] + 1] = g[q] + W[q];
    /* populations -> central moments: z lines, then y, then x */
    for (int x = 0; x < 3; ++x)
        for (int y = 0; y < 3; ++y) {
            double l[3] = {K[x][y][0], K[x][y][1], K[x][y][2]};
            forward_line(l, u[2]);
            for (int k = 0; k < 3; ++k) K[x][y][k] = l[k];
        }
    for (int x = 0; x < 3; ++x)
        for (int c = 0; c < 3; ++c) {
            double l[3] = {K[x][0][c], K[x][1][c], K[x][2][c]};
            forward_line(l, u[1]);
            for (int k = 0; k < 3; ++k) K[x][k][c] = l[k];
        }
    for (int b = 0; b < 3; ++b)
        for (int c = 0; c < 3; ++c) {
            double l[3] = {K[0][b][c], K[1][b][c], K[2][b][c]};
            forward_line(l, u[0]);
            for (int k = 0; k < 3; ++k) K[k][b][c] = l[k];
        }
    /* second-order cumulants equal the central moments; relax the five
     * deviatoric combinations with omega_s and the trace with omega_b towards
     * rho*cs^2 per diagonal entry */
    double kxx = K[2][0][0], kyy = K[0][2][0], kzz = K[0][0][2];
    if (c18 > 0.0)
        omega_s = smagorinsky_rate(omega_s, c18, rho, kxx - rho / 3.0, kyy - rho / 3.0, kzz - rho / 3.0, K[1][1][0],
                                   K[1][0][1], K[0][1][1]);
    double d1 = (1.0 - omega_s) * (kxx - kyy);
    double d2 = (1.0 - omega_s) * (kxx - kzz);
    double tr = kxx + kyy + kzz;
    tr = tr + omega_b * (rho - tr);
    double s[6];
    s[0] = (d1 + d2 + tr) / 3.0;
    s[1] = s[0] - d1;
    s[2] = s[0] - d2;
    s[3] = (1.0 - omega_s) * K[1][1][0];
    s[4] = (1.0 - omega_s) * K[1][0][1];
    s[5] = (1.0 - omega_s) * K[0][1][1];
    /* all higher cumulants relax to their zero equilibrium with rate 1, so the
     * post-collision central moments are Gaussian (Isserlis) pairings of the
     * normalised second-order ones; odd orders vanish */
    double sxx = s[0] / rho, syy = s[1] / rho, szz = s[2] / rho;
    double sxy = s[3] / rho, sxz = s[4] / rho, syz = s[5] / rho;
    memset(K, 0, sizeof K);
    K[0][0][0] = rho;
    K[2][0][0] = s[0];
    K[0][2][0] = s[1];
    K[0][0][2] = s[2];
    K[1][1][0] = s[3];
    K[1][0][1] = s[4];
    K[0][1][1] = s[5];
    K[2][2][0] = rho * (sxx * syy + 2.0 * sxy * sxy);
    K[2][0][2] = rho * (sxx * szz + 2.0 * sxz * sxz);
    K[0][2][2] = rho * (syy * szz + 2.0 * syz * syz);
    K[2][1][1] = rho * (sxx * syz + 2.0 * sxy * sxz);
    K[1][2][1] = rho * (syy * sxz + 2.0 * sxy * syz);
    K[1][1][2] = rho * (szz * sxy + 2.0 * sxz * syz);
    K[2][2][2] = rho * (sxx * syy * szz + 2.0 * (sxx * syz * syz + syy * sxz * sxz + szz * sxy * sxy) +
                        8.0 * sxy * sxz * syz);
    /* central moments -> populations: x lines, then y, then z */
    for (int b = 0; b < 3; ++b)
        for (int c = 0; c < 3; ++c) {
            double l[3] = {K[0][b][c], K[1][b][c], K[2][b][c]};
            backward_line(l, u[0]);
            for (int k = 0; k < 3; ++k) K[k][b][c] = l[k];
        }
    for (int x = 0; x < 3; ++x)
        for (int c = 0; c < 3; ++c) {
            double l[3] = {K[x][0][c], K[x][1][c], K[x][2][c]};
            backward_line(l, u[1]);
            for (int k = 0; k < 3; ++k) K[x][k][c] = l[k];
        }
    for (int x = 0; x < 3; ++x)
        for (int y = 0; y < 3; ++y) {
            double l[3] = {K[x][y][0], K[x][y][1], K[x][y][2]};
            backward_line(l, u[2]);
            for (int k = 0; k < 3; ++k) K[x][y][k] = l[k];
        }
    for (int q = 0; q < Q; ++q) g[q] = K[CV[q][0] + 1][CV[q][1] + 1][CV[q][2] + 1] - W[q];
}

static void collide_cell(double *g, double omega_s, double omega_b) { collide_cell_sgs(g, omega_s, omega_b, 0.0); }

void ako_collide_cells(double *g, int64_t n, double omega_s, double omega_b) {
    init_tables();
    for (int64_t i = 0; i < n; ++i) collide_cell(g + Q * i, omega_s, omega_b);
}

void ako_collide_cells_sgs(double *g, int64_t n, double omega_s, double omega_b, double c18) {
    init_tables();
    for (int64_t i = 0; i < n; ++i) collide_cell_sgs(g + Q * i, omega_s, omega_b, c18);
}

#define IDX(x, y, z) ((((int64_t)(x) * NY + (y)) * NZ + (z)) * Q)

/* Pull-stream every interior cell from src, collide, write dst (the reference's
 * "stream_collide" kernel; solid cells are updated too, as the generated kernel
 * does, and their values are never read by the fluid). */
void ako_stream_collide_sgs(const double *src, double *dst, int nx, int ny, int nz, double omega_s,
                            double omega_b, double c18, int threads) {
    init_tables();
    const int NY = ny + 2, NZ = nz + 2;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for collapse(2) schedule(static)
#endif
    for (int x = 1; x <= nx; ++x)
        for (int y = 1; y <= ny; ++y)
            for (int z = 1; z <= nz; ++z) {
                double g[Q];
                for (int q = 0; q < Q; ++q) g[q] = src[IDX(x - CV[q][0], y - CV[q][1], z - CV[q][2]) + q];
                collide_cell_sgs(g, omega_s, omega_b, c18);
                memcpy(dst + IDX(x, y, z), g, sizeof g);
            }
}

void ako_stream_collide(const double *src, double *dst, int nx, int ny, int nz, double omega_s,
                        double omega_b, int threads) {
    ako_stream_collide_sgs(src, dst, nx, ny, nz, omega_s, omega_b, 0.0, threads);
}

/* Only the "collide" half, in place (refined levels order collide, stream). */
void ako_collide(double *pdf, int nx, int ny, int nz, double omega_s, double omega_b, int threads) {
    init_tables();
    const int NY = ny + 2, NZ = nz + 2;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for collapse(2) schedule(static)
#endif
    for (int x = 1; x <= nx; ++x)
        for (int y = 1; y <= ny; ++y)
            for (int z = 1; z <= nz; ++z) collide_cell(pdf + IDX(x, y, z), omega_s, omega_b);
}

/* Only the pull-stream half, src -> dst, over interior cells. */
void ako_stream(const double *src, double *dst, int nx, int ny, int nz) {
    init_tables();
    const int NY = ny + 2, NZ = nz + 2;
    for (int x = 1; x <= nx; ++x)
        for (int y = 1; y <= ny; ++y)
            for (int z = 1; z <= nz; ++z)
                for (int q = 0; q < Q; ++q)
                    dst[IDX(x, y, z) + q] = src[IDX(x - CV[q][0], y - CV[q][1], z - CV[q][2]) + q];
}

/* Periodic ghost copy along the axes whose flag is set (all ghost rows of the
 * other axes included, as a full-slab copy does). */
void ako_sync_periodic(double *pdf, int nx, int ny, int nz, int px, int py, int pz) {
    const int NX = nx + 2, NY = ny + 2, NZ = nz + 2;
    (void)NX;
    if (px)
        for (int y = 0; y < NY; ++y)
            for (int z = 0; z < NZ; ++z) {
                memcpy(pdf + IDX(0, y, z), pdf + IDX(nx, y, z), Q * sizeof(double));
                memcpy(pdf + IDX(nx + 1, y, z), pdf + IDX(1, y, z), Q * sizeof(double));
            }
    if (py)
        for (int x = 0; x < NX; ++x)
            for (int z = 0; z < NZ; ++z) {
                memcpy(pdf + IDX(x, 0, z), pdf + IDX(x, ny, z), Q * sizeof(double));
                memcpy(pdf + IDX(x, ny + 1, z), pdf + IDX(x, 1, z), Q * sizeof(double));
            }
    if (pz)
        for (int x = 0; x < NX; ++x)
            for (int y = 0; y < NY; ++y) {
                memcpy(pdf + IDX(x, y, 0), pdf + IDX(x, y, nz), Q * sizeof(double));
                memcpy(pdf + IDX(x, y, nz + 1), pdf + IDX(x, y, 1), Q * sizeof(double));
            }
}

/* Tensor-product equilibrium minus the weights, for n cells (rho, u given). */
static void equilibrium_g(double rho, const double *u, double *g) {
    for (int q = 0; q < Q; ++q) {
        double p = rho;
        for (int a = 0; a < 3; ++a) {
            double v = u[a];
            int c = CV[q][a];
            p *= c == 0 ? 2.0 / 3.0 - v * v : 0.5 * (1.0 / 3.0 + v * v + c * v);
        }
        g[q] = p - W[q];
    }
}

void ako_equilibrium(double *g, const double *rho, const double *u, int64_t n) {
    init_tables();
    for (int64_t i = 0; i < n; ++i) equilibrium_g(rho[i], u + 3 * i, g + Q * i);
}

/* Macroscopic rho, u of n cells of zero-centred populations. */
void ako_macros(const double *g, double *rho, double *u, int64_t n) {
    init_tables();
    for (int64_t i = 0; i < n; ++i) {
        double d = 0.0, j[3] = {0.0, 0.0, 0.0};
        for (int q = 0; q < Q; ++q) {
            d += g[Q * i + q];
            for (int a = 0; a < 3; ++a) j[a] += CV[q][a] * g[Q * i + q];
        }
        double r = 1.0 + d;
        rho[i] = r;
        for (int a = 0; a < 3; ++a) u[3 * i + a] = j[a] / r;
    }
}

/* ---- boundaries over link lists: link = (x, y, z, d) in padded coordinates,
 * the fluid cell x and the direction d towards the boundary cell x + c_d ---- */

/* NoSlipLinearBouzidi; q < 0 is the half-way fallback. */
void ako_bouzidi(double *pdf, int nx, int ny, int nz, int64_t n, const int32_t *links, const double *qs) {
    init_tables();
    const int NY = ny + 2, NZ = nz + 2;
    (void)nx;
    for (int64_t i = 0; i < n; ++i) {
        int x = links[4 * i], y = links[4 * i + 1], z = links[4 * i + 2], d = links[4 * i + 3];
        double q = qs[i];
        double f_xf = pdf[IDX(x, y, z) + d];
        double f_xf_inv = pdf[IDX(x, y, z) + INV[d]];
        double d_x2f = pdf[IDX(x - CV[d][0], y - CV[d][1], z - CV[d][2]) + d];
        double v;
        if (q >= 0.5)
            v = (0.5 * (f_xf + f_xf_inv * (2.0 * q - 1.0))) / q;
        else if (q > 0.0)
            v = 2.0 * q * f_xf + (1.0 - 2.0 * q) * d_x2f;
        else
            v = f_xf;
        pdf[IDX(x + CV[d][0], y + CV[d][1], z + CV[d][2]) + INV[d]] = v;
    }
}

/* Velocity bounce-back with the compressible density factor of the fluid cell. */
void ako_ubb(double *pdf, int nx, int ny, int nz, int64_t n, const int32_t *links, const double *vel) {
    init_tables();
    const int NY = ny + 2, NZ = nz + 2;
    (void)nx;
    for (int64_t i = 0; i < n; ++i) {
        int x = links[4 * i], y = links[4 * i + 1], z = links[4 * i + 2], d = links[4 * i + 3];
        const double *g = pdf + IDX(x, y, z);
        double drho = 0.0;
        for (int q = 0; q < Q; ++q) drho += g[q];
        double rho = drho + 1.0;
        double cu = CV[d][0] * vel[0] + CV[d][1] * vel[1] + CV[d][2] * vel[2];
        double term = 6.0 * cu * W[d];
        pdf[IDX(x + CV[d][0], y + CV[d][1], z + CV[d][2]) + INV[d]] = g[d] - term * rho;
    }
}

/* ExtrapolationOutflow, Geier et al. 2015 eq. (F.1) as configured at
 * solver.py:133-135: the incoming population on the boundary cell is advected
 * outwards with the speed of sound c = cs*dt/dx = sqrt(1/3) by one first-order
 * upwind step,  f_b(t+1) = c f_n(t) + (1-c) f_b(t),  where f_n is the same
 * population on the fluid neighbour x_b - n of the boundary cell.  Each link
 * keeps two values: state[2i] = f_n of the previous step and state[2i+1] =
 * f_b of the previous step; both start at the zero-centred equilibrium of the
 * initial density and velocity.  (This two-value form, and its start from the
 * zero-centred equilibrium, are the ones that reproduce the reference's
 * plane-wave probe record docs/verification_stage1_20261106/acoustics/
 * extrapolation.csv to rounding.) */
static const double CS = 0.57735026918962576451;
static const double ONE_MINUS_CS = 0.42264973081037423549;

void ako_outflow(double *pdf, int nx, int ny, int nz, int64_t n, const int32_t *links, const int *normal,
                 double *state) {
    init_tables();
    const int NY = ny + 2, NZ = nz + 2;
    (void)nx;
    for (int64_t i = 0; i < n; ++i) {
        int x = links[4 * i], y = links[4 * i + 1], z = links[4 * i + 2], d = links[4 * i + 3];
        int inv = INV[d];
        int tx = x + CV[d][0] - normal[0], ty = y + CV[d][1] - normal[1], tz = z + CV[d][2] - normal[2];
        double neighbour = pdf[IDX(tx, ty, tz) + inv];
        double *s = state + 2 * i;
        double v = CS * s[0] + ONE_MINUS_CS * s[1];
        s[0] = neighbour;
        s[1] = v;
        pdf[IDX(x + CV[d][0], y + CV[d][1], z + CV[d][2]) + inv] = v;
    }
}

/* ---- characteristic farfield, restating farfield.py:144-206 ---- */
static void macro_at(const double *pdf, int NY, int NZ, int x, int y, int z, double *rho, double *u) {
    const double *g = pdf + IDX(x, y, z);
    double d = 0.0, j[3] = {0.0, 0.0, 0.0};
    for (int q = 0; q < Q; ++q) {
        d += g[q];
        for (int a = 0; a < 3; ++a) j[a] += CV[q][a] * g[q];
    }
    *rho = 1.0 + d;
    for (int a = 0; a < 3; ++a) u[a] = j[a] / *rho;
}

static double feq_dir(double r, const double *v, const int *c) {
    double p = r;
    for (int a = 0; a < 3; ++a) {
        double cc = (double)c[a], q = v[a];
        p *= 2.0 / 3.0 - q * q + (1.5 * q * q - 0.5) * cc * cc + cc * q / 2.0;
    }
    return p;
}

/*
 * mode 0: inflow face (n.U < 0), incoming invariant fixed to n.U;
 * mode 1: outflow face, incoming invariant evolved by the trapezoidal rule with
 *         the linearised transverse term (state: incoming, derivative);
 * mode 2: glancing face (n.U = 0), initial invariant traced along U (state:
 *         clock; initial field `initial`, interior-shaped (nx, ny, nz)).
 * edge/wrap are per link and per axis as built by the reference's init
 * callback (farfield.py:56-73).
 */
void ako_farfield(double *pdf, int nx, int ny, int nz, int64_t n, const int32_t *links, const int *normal,
                  const double *vel, double density, int mode, double *incoming, double *derivative,
                  int64_t *clock, const int32_t *edge, const int32_t *wrap, const double *initial,
                  const int *periodic) {
    init_tables();
    const int NY = ny + 2, NZ = nz + 2;
    const int shape[3] = {nx, ny, nz};
    double nrm = sqrt((double)(normal[0] * normal[0] + normal[1] * normal[1] + normal[2] * normal[2]));
    double nh[3] = {normal[0] / nrm, normal[1] / nrm, normal[2] / nrm};
    double un_inf = nh[0] * vel[0] + nh[1] * vel[1] + nh[2] * vel[2];
    double ut_inf[3], P[3][3];
    for (int a = 0; a < 3; ++a) {
        ut_inf[a] = vel[a] - un_inf * nh[a];
        for (int b = 0; b < 3; ++b) P[a][b] = (a == b ? 1.0 : 0.0) - nh[a] * nh[b];
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < n; ++i) {
        int x = links[4 * i], y = links[4 * i + 1], z = links[4 * i + 2], d = links[4 * i + 3];
        int inv = INV[d];
        int foot[3];
        int cell[3] = {x, y, z};
        for (int a = 0; a < 3; ++a) foot[a] = cell[a] + CV[d][a] - normal[a] + wrap[3 * i + a];
        double rho, u[3];
        macro_at(pdf, NY, NZ, foot[0], foot[1], foot[2], &rho, u);
        double un = nh[0] * u[0] + nh[1] * u[1] + nh[2] * u[2];
        double lr = log(rho / density);
        double rm = un - CS * lr, rp = un + CS * lr;
        double F = 0.0, value;
        if (mode == 1) {
            for (int a = 0; a < 3; ++a) {
                if (ut_inf[a] == 0.0 && P[a][0] == 0.0 && P[a][1] == 0.0 && P[a][2] == 0.0) continue;
                int e = edge[3 * i + a];
                int off1 = e == -1 ? 1 : -1;
                int off2 = e == 0 ? 1 : -2 * e;
                double c0 = 1.5 * e;
                double c1 = e == 0 ? -0.5 : -2.0 * e;
                double c2 = e == 0 ? 0.5 : 0.5 * e;
                int s1[3] = {foot[0], foot[1], foot[2]}, s2[3] = {foot[0], foot[1], foot[2]};
                s1[a] += off1;
                s2[a] += off2;
                double r1, v1[3], r2, v2[3];
                macro_at(pdf, NY, NZ, s1[0], s1[1], s1[2], &r1, v1);
                macro_at(pdf, NY, NZ, s2[0], s2[1], s2[2], &r2, v2);
                double du[3];
                for (int b = 0; b < 3; ++b) du[b] = c0 * u[b] + c1 * v1[b] + c2 * v2[b];
                double rm1 = nh[0] * v1[0] + nh[1] * v1[1] + nh[2] * v1[2] - CS * log(r1 / density);
                double rm2 = nh[0] * v2[0] + nh[1] * v2[1] + nh[2] * v2[2] - CS * log(r2 / density);
                F += un_inf * (P[a][0] * du[0] + P[a][1] * du[1] + P[a][2] * du[2]) -
                     ut_inf[a] * (c0 * rm + c1 * rm1 + c2 * rm2);
            }
            value = incoming[i] + (F + derivative[i]) / 2.0;
        } else if (mode == 2) {
            /* one linear interpolation of the saved initial invariant at the
             * total shift U*clock, along the axes where U is non-zero */
            double sum = 0.0;
            int axes[3], na = 0;
            for (int a = 0; a < 3; ++a)
                if (vel[a] != 0.0) axes[na++] = a;
            double target[3], fraction[3];
            int lower[3];
            for (int a = 0; a < 3; ++a) {
                /* foot cell in interior coordinates, shifted back along U */
                target[a] = (double)(foot[a] - 1) - vel[a] * (double)clock[i];
                lower[a] = (int)floor(target[a]);
                fraction[a] = target[a] - lower[a];
            }
            for (int bits = 0; bits < (1 << na); ++bits) {
                double weight = 1.0;
                int coord[3], valid = 1;
                for (int a = 0; a < 3; ++a) coord[a] = foot[a] - 1; /* interior coordinates */
                for (int k = 0; k < na; ++k) {
                    int a = axes[k], bit = (bits >> k) & 1;
                    int kk = lower[a] + bit;
                    weight *= bit ? fraction[a] : 1.0 - fraction[a];
                    if (periodic[a]) {
                        int m = kk % shape[a];
                        coord[a] = m < 0 ? m + shape[a] : m;
                    } else {
                        coord[a] = kk < 0 ? 0 : (kk > shape[a] - 1 ? shape[a] - 1 : kk);
                        if (kk < 0 || kk >= shape[a]) valid = 0;
                    }
                }
                double sample = initial[((int64_t)coord[0] * ny + coord[1]) * nz + coord[2]];
                sum += weight * (valid ? sample : 0.0);
            }
            value = un_inf + sum;
        } else {
            value = un_inf;
        }
        double unb = (rp + value) / 2.0;
        double rhob = density * exp((rp - value) / (2.0 * CS));
        double ub[3];
        for (int a = 0; a < 3; ++a) {
            double tangential = unb >= 0.0 ? u[a] - nh[a] * un : vel[a] - nh[a] * un_inf;
            ub[a] = nh[a] * unb + tangential;
        }
        const int *ci = CV[inv];
        double ghost = pdf[IDX(foot[0], foot[1], foot[2]) + inv] + feq_dir(rhob, ub, ci) - feq_dir(rho, u, ci);
        pdf[IDX(x + CV[d][0], y + CV[d][1], z + CV[d][2]) + inv] = ghost;
        if (mode == 1) {
            incoming[i] = value;
            derivative[i] = F;
        }
        if (mode == 2) clock[i] += 1;
    }
}

/* ---- momentum exchange (solver.py:204-250): per link, F += c_d (g_out + g_in)
 * with g_out = pdf[x](d) and g_in = pdf[x + c_d](inv d); Mz about the origin of
 * the lattice-unit frame given by (ox, oy) = storage origin / dx ---- */
void ako_loads(const double *pdf, int nx, int ny, int nz, int64_t n, const int32_t *links, double ox,
               double oy, double *out) {
    init_tables();
    const int NY = ny + 2, NZ = nz + 2;
    (void)nx;
    double f[3] = {0.0, 0.0, 0.0}, mz = 0.0, mass = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        int x = links[4 * i], y = links[4 * i + 1], z = links[4 * i + 2], d = links[4 * i + 3];
        double go = pdf[IDX(x, y, z) + d];
        double gi = pdf[IDX(x + CV[d][0], y + CV[d][1], z + CV[d][2]) + INV[d]];
        double v = go + gi;
        double lf[3] = {CV[d][0] * v, CV[d][1] * v, CV[d][2] * v};
        for (int a = 0; a < 3; ++a) f[a] += lf[a];
        double rx = (double)(x - 1) + 0.5 + ox, ry = (double)(y - 1) + 0.5 + oy;
        mz += rx * lf[1] - ry * lf[0];
        mass += gi - go;
    }
    out[0] = f[0];
    out[1] = f[1];
    out[2] = f[2];
    out[3] = mz;
    out[4] = mass;
}
