/*
 * aerokinetic_gb300.h -- C ABI of the GB300 engine for AeroKinetic's uniform
 * D3Q27 cumulant lattice-Boltzmann step.
 *
 * The reference (Bulbulator72/Aerokinetic 0.5.3, Python) drives a lbmpy
 * LatticeBoltzmannStep through a handful of private calls; each entry point
 * below replaces one of them (reference paths are relative to that project):
 *
 *   ak_case_create      LatticeBoltzmannStep construction and boundary set-up,
 *                       src/aerokinetic/solver.py:58-91 and 124-155 (solid
 *                       flags, cut links, Bouzidi q with the half-way fallback,
 *                       UBB/ExtrapolationOutflow or the characteristic farfield
 *                       of src/aerokinetic/farfield.py:209-224)
 *   ak_init_perturbed   Solver._initialize, solver.py:157-202
 *   ak_init_fields      LatticeBoltzmannStep.set_pdf_fields_from_macroscopic_values
 *                       with caller-supplied rho/u (solver.py:202)
 *   ak_step             the step body, solver.py:256-261 (_sync_src,
 *                       boundary_handling, run_kernel(stream_collide), swap),
 *                       with the loads of Solver._loads, solver.py:204-250
 *   ak_diagnostics      Solver.diagnostics, solver.py:281-297
 *   ak_macros           LatticeBoltzmannStep.post_run + gather_array of the
 *                       density/velocity fields (solver.py:283-286, 318-319)
 *   ak_get_pdf /        data_handling.cpu_arrays[pdf] reads and writes used by
 *   ak_set_pdf          the checkpoint module (checkpoint.py:20-68)
 *   ak_get_wall_links   boundary_handling index lists of the walls
 *                       (walls.py:51-66, solver.py:218-226)
 *
 * Conventions.  All functions return 0 (AK_OK) or an AK_ERR_* code and leave
 * a message for ak_last_error.  Populations cross the ABI as double, in the
 * reference's layout: (nx, ny, nz, 27) C order, interior cells only,
 * zero-centred g = f - w, lbmpy's D3Q27 direction order.  Device memory is
 * allocated and owned by the case; every call on one case is stream-ordered on
 * the case's own CUDA stream and returns after its results are on the host.
 * One case may be used by one host thread at a time.
 */
#ifndef AEROKINETIC_GB300_H
#define AEROKINETIC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AK_OK 0
#define AK_ERR_INVALID 1     /* bad argument; maps to ValueError */
#define AK_ERR_CUDA 2        /* CUDA runtime failure */
#define AK_ERR_NOMEM 3       /* device allocation failed; maps to MemoryError */
#define AK_ERR_NONFINITE 4   /* non-finite state; maps to NumericalFailure */
#define AK_ERR_GUARD 5       /* local Mach or density guard; maps to NumericalFailure */
#define AK_ERR_GEOMETRY 6    /* a cut link without a polygon crossing */

#define AK_FARFIELD_LEGACY 0          /* UBB + ExtrapolationOutflow (solver.py:130-135) */
#define AK_FARFIELD_CHARACTERISTIC 1  /* characteristic_transport_v1 (farfield.py) */
#define AK_FARFIELD_EXTERIOR 2        /* exterior_regularized_fd_v1 (exterior.py): the ghost layer is an
                                         auxiliary ring rebuilt each step from a predicted state */

#define AK_STORAGE_F64 0  /* plain form: FP64 storage and arithmetic */
#define AK_STORAGE_F32 1  /* FP32 arithmetic, FP32 (f - w) storage */
#define AK_STORAGE_F16 2  /* FP32 arithmetic, FP16 storage of (f - f_eq(1, U)) / w */
#define AK_STORAGE_DF64 3 /* 8-byte storage as FP32 pairs, collision in double-float (48-bit) arithmetic,
                             boundaries and refinement transfers in FP64 */

typedef struct ak_case ak_case;

typedef struct {
    int32_t nx, ny, nz;          /* interior lattice; z is periodic */
    double origin_x, origin_y;   /* plan origin (chord units), solver.py:39-40 */
    double dx;                   /* plan dx = 1 / cells_per_chord */
    double omega_shear;          /* plan relaxation rate */
    double omega_bulk;           /* 1.0 for the uniform solver */
    double speed;                /* freestream lattice speed along +x */
    int32_t farfield;            /* AK_FARFIELD_* */
    int32_t storage;             /* AK_STORAGE_* */
    int32_t n_elements;          /* number of polygons (wall elements) */
    const int32_t *element_sizes;/* vertices per polygon */
    const double *polygon_xy;    /* all vertices, (x, y) pairs, normalised frame */
    double smagorinsky;          /* Smagorinsky constant C of sgs="smagorinsky" (solver.py:74-77), 0 for
                                    molecular viscosity; uniform legacy/characteristic cases only */
} ak_case_desc;

typedef struct {
    int64_t cells;          /* nx * ny * nz */
    int64_t fluid_cells;
    int64_t wall_keys;      /* distinct (column, planar direction) cut links */
    int64_t wall_links;     /* wall_keys * nz * 3 */
    int64_t outer_links;    /* links into the outer ghost ring */
    int64_t fallback_links; /* 3-D links using the half-way fallback */
    int64_t device_bytes;   /* bytes of device memory held by the case */
    int32_t row_pitch;      /* elements between consecutive x rows */
    int32_t storage;
} ak_case_info;

/* solver.py:58-155.  Builds the case on the current CUDA device. */
int ak_case_create(const ak_case_desc *desc, ak_case **out);
int ak_case_destroy(ak_case *c);
int ak_case_get_info(const ak_case *c, ak_case_info *info);

/* solver.py:157-202: rho = 1, u = (U, u_y, u_z) with the divergence-free
 * perturbation of amplitude amp (= perturbation * U), phases phase_y/phase_z,
 * Gaussian envelope about the rotated leading edge (lead_x, lead_y), span in
 * chord units; solid cells at rest. */
int ak_init_perturbed(ak_case *c, double amp, double phase_y, double phase_z, double lead_x,
                      double lead_y, double span);
/* set_pdf_fields_from_macroscopic_values with host rho (nx*ny*nz) and u (*3). */
int ak_init_fields(ak_case *c, const double *rho, const double *u);

/* Advance nsteps steps.  If loads != NULL the last step samples the
 * momentum-exchange loads before streaming (solver.py:258-259) into
 * loads[n_elements * 5] = (Fx, Fy, Fz, Mz, incoming-minus-outgoing mass) per
 * element, in lattice units, Mz about the normalised frame's origin. */
int ak_step(ak_case *c, int32_t nsteps, double *loads);
/* ak_step with loads that allocates no device memory, for callers that
 * cannot allocate once running (a host whose memory pool already holds the
 * GPU's free memory, a fixed device budget, a plugin host that forbids
 * allocation after start-up): the per-block partial sums of the loads live
 * in a static device array of 131072 doubles (1 MiB, held by every GPU that
 * loads the library).  No counterpart in the reference.  The first call on a
 * device looks up the array's device address, with the case's device
 * current.  Steps run eagerly (no graph replay).  Cases whose wall links
 * need more partial sums than the array holds get AK_ERR_INVALID before
 * anything is launched: a rejected call leaves the case unchanged.  All
 * calls share the array: calls that overlap on the GPU (other cases on
 * other streams) race. */
int ak_step_loads_static(ak_case *c, int32_t nsteps, double *loads);
int64_t ak_steps_done(const ak_case *c);
/* Kernels the case has issued while stepping (for launch accounting). */
int64_t ak_kernel_launches(const ak_case *c);
/* The case's CUDA stream (cudaStream_t), for callers that order their own work
 * after the case's or time it with their own events. */
void *ak_case_stream(const ak_case *c);
/* ak_step without loads, timed with CUDA events on the case's stream:
 * ms[0] whole interval, ms[1] stream-collide kernels, ms[2] wall kernels,
 * ms[3] outer-boundary kernels (milliseconds, summed over the steps).  No
 * counterpart in the reference; it exists for measurement. */
int ak_step_timed(ak_case *c, int32_t nsteps, double *ms);

/* diag[0] = local Mach max over fluid cells, diag[1] = mean density of fluid
 * cells, diag[2] = max |rho - 1|, diag[3] = min rho, diag[4] = 1 if every
 * fluid value is finite.  Returns AK_ERR_NONFINITE / AK_ERR_GUARD like
 * solver.py:289-294 after filling diag. */
int ak_diagnostics(ak_case *c, double *diag);

/* rho (nx*ny*nz) and u (nx*ny*nz*3) of the current state, to host memory. */
int ak_macros(ak_case *c, double *rho, double *u);
int ak_get_pdf(ak_case *c, double *pdf);
int ak_set_pdf(ak_case *c, const double *pdf);

/* History of the outer boundary for checkpoints (checkpoint.py:32-135 keeps
 * lbmpy's boundary index arrays for the same reason): n_links outer links,
 * rows[4 k .. 4 k + 3] = (x, y, z, direction) of link k in interior
 * coordinates; values[0] = 1 once the boundary data are prepared, then for the
 * characteristic farfield incoming[n], derivative[n], glancing clock[n],
 * initial invariant rows lo[nx * nz], hi[nx * nz]; for the legacy boundary the
 * ExtrapolationOutflow state (neighbour, boundary value) of each outflow link.
 * ak_set_boundary_state refuses rows that differ from the case's own. */
int ak_boundary_state_size(ak_case *c, int64_t *n_links, int64_t *n_values);
int ak_get_boundary_state(ak_case *c, int32_t *rows, double *values);
int ak_set_boundary_state(ak_case *c, const int32_t *rows, const double *values);
/* exterior_regularized_fd_v1 bookkeeping (solver.py:262-271, 299-309):
 * out[0..3] = the last step's exterior source (mass, momentum x/y/z: the
 * rebuilt ring populations minus the streamed ones, exterior.py:195-200),
 * out[4..7] their running sums, out[8] the last step's wall mass exchange
 * (incoming minus outgoing over all wall links), out[9] its running sum,
 * out[10] the last step's reconstruction moment error (the largest departure
 * of a rebuilt ring cell's mass or momentum from its predicted rho, rho u,
 * exterior.py:168-170).  out holds 11 doubles.
 * An exterior case stores post-collision populations (ak_get_pdf returns
 * them); its initial state is prepared by ak_init_perturbed/ak_init_fields,
 * and its checkpoint state (ring populations, ring-band macros, the initial
 * incoming invariant of the glancing rows, these sums) travels through
 * ak_get/set_boundary_state with no link rows. */
int ak_exterior_report(ak_case *c, double *out);
/* The case's two population arrays in device memory, for zero-copy views
 * (e.g. torch tensors through __cuda_array_interface__): current holds the
 * state ak_get_pdf returns, other the second copy.  Layout [q][z][y][x] with
 * dims = (27, nz, ny + 2, row pitch), x and y offset by one ghost layer;
 * element_bytes 8 (f64 doubles, df64 (hi, lo) float pairs), 4 (f32) or 2
 * (f16, (f - f_eq(1, U)) / w).  Valid until the next step swaps the copies. */
int ak_case_buffers(ak_case *c, void **current, void **other, int64_t *dims, int32_t *element_bytes);
/* Step counter of a restored case (Solver.steps after restore_checkpoint,
 * checkpoint.py:113). */
int ak_set_steps_done(ak_case *c, int64_t steps);

/* Stationarity residuals (convergence.py:58-96) without a host gather: over
 * the case's owned fluid cells (the whole interior of a uniform case; for a
 * two-level case's levels, the coarse cells outside the fine box and the
 * physical fine block), with a device snapshot of (rho, j * inv_speed) per
 * cell, out[9] = sum over cells of ((current - snapshot) * inv_dt)^2 for the
 * four components, their max |.|, and the number of cells; the snapshot then
 * takes the current values.  reset != 0 only takes the snapshot. */
int ak_residuals(ak_case *c, double inv_speed, double inv_dt, int32_t reset, double *out);
/* The snapshot as 4 doubles per owned cell (count returned; data may be null):
 * write = 0 copies it out, write != 0 replaces it (checkpoints). */
int ak_residual_snapshot(ak_case *c, int32_t write, double *data, int64_t *count);

/* Solid flags of the interior columns (nx*ny, x-major like the reference's
 * _solid_xy): 0 fluid, k+1 inside element k. */
int ak_get_flags(ak_case *c, uint8_t *flags);
/* Distinct wall keys: rows[4k..4k+3] = (element, x, y, direction index of the
 * planar link), q[k] the Bouzidi fraction (-1 = half-way fallback). */
int ak_get_wall_links(ak_case *c, int32_t *rows, double *q);

/* ---- two-level (2:1) refined case: refined_solver.py:115-345 and
 * interface.py:133-352.  One coarse lattice with the legacy outer boundary
 * and a fine block (2x resolution, walls on the fine level) over the box;
 * each coarse step runs two fine steps with time-interpolated donors,
 * face-flux reflux and restriction. */
typedef struct ak_refined ak_refined;

typedef struct {
    ak_case_desc coarse;         /* the uniform plan of the coarse level (legacy farfield) */
    double tau_shear, tau_bulk;  /* coarse relaxation times (refined_solver.py:77-78) */
    double dt_coarse;            /* coarse time step in convective units */
    double span;                 /* periodic span in chord units */
    int32_t box_lower[3], box_upper[3];  /* fine box in coarse cells; z spans the whole span */
    int32_t fine_storage;        /* AK_STORAGE_* of the fine level (the walls' level): -1 = the coarse
                                    level's; AK_STORAGE_F32 under an AK_STORAGE_F16 coarse level */
} ak_refined_desc;

/* RefinedSolver construction (refined_solver.py:116-162). */
int ak_refined_create(const ak_refined_desc *desc, ak_refined **out);
int ak_refined_destroy(ak_refined *r);
/* initialize_flow (refined_solver.py:224-269): free stream everywhere, the
 * seeded perturbation on both levels, covered coarse cells restricted from
 * the fine level, outflow history from that state. */
int ak_refined_init_perturbed(ak_refined *r, double amp, double phase_y, double phase_z, double lead_x,
                              double lead_y);
/* nsteps coarse steps (PeriodicRefinedBox._step_once, interface.py:311-352);
 * loads[n_elements * 5] = fine-lattice (Fx, Fy, Fz, Mz, mass) of the last
 * coarse step summed over its two fine steps (walls.py:68-95), Mz about the
 * normalised frame's origin in fine lattice units.  The steps' kernels are
 * captured once per buffer parity into CUDA graphs and replayed, up to four
 * steps per graph where the coarse pass runs on its own branch (each step's
 * first fine step beside the previous step's coarse pass). */
int ak_refined_step(ak_refined *r, int32_t nsteps, double *loads);
/* ak_refined_step that also returns, with one synchronisation, what the
 * budget of the last step needs (refined_solver.py:329-339): outer[8] as
 * ak_refined_outer_flux, stats[16] as ak_refined_integrals of the state the
 * step leaves, but with the two maxima (diagnostics only) left 0.  With stats
 * every step computes these integrals, as the reference's step does; in the
 * FP64-arithmetic forms the coarse level's come out of the fused
 * stream-collide pass itself.  The sums are exact fixed-point integer sums of
 * each cell's values rounded to 2^-50 (a cell with a value of magnitude 256
 * or more, or a population of magnitude 1 or more, counts as non-finite).
 * Needs ak_refined_track_budget on; outer or stats may be NULL. */
int ak_refined_step_budget(ak_refined *r, int32_t nsteps, double *loads, double *outer, double *stats);
int64_t ak_refined_steps_done(const ak_refined *r);
/* With enable != 0, every following step also measures the inflow through
 * the outer x and y faces of the coarse lattice after its boundaries
 * (refined_solver.py:274-278, the samplers of refined_solver.py:215-222). */
int ak_refined_track_budget(ak_refined *r, int32_t enable);
/* out[0..3] = inflow (mass, jx, jy, jz) of the last tracked step, coarse
 * lattice units times dx^3: the reference's _interval_external_in before its
 * momentum is scaled to common velocity units; out[4..7] = its sum over the
 * tracked steps since initialisation (cumulative_external_in,
 * refined_solver.py:342). */
int ak_refined_outer_flux(ak_refined *r, double *out);
/* out[n_elements * 5] = fine-lattice (Fx, Fy, Fz, Mz, mass) summed over every
 * step since initialisation (cumulative_wall_impulse and
 * cumulative_wall_mass_exchange, refined_solver.py:340-341). */
int ak_refined_cumulative_loads(ak_refined *r, double *out);
/* Restores a checkpoint's step count and running sums (refined_checkpoint.py):
 * cumulative_loads[n_elements * 5] as ak_refined_cumulative_loads returns
 * them, cumulative_outer[4] as out[4..7] of ak_refined_outer_flux. */
int ak_refined_restore_counters(ak_refined *r, int64_t steps, const double *cumulative_loads,
                                const double *cumulative_outer);
/* Per-level statistics for conserved_integrals and diagnostics
 * (refined_solver.py:291-299, 347-361): out[0..7] coarse cells outside the
 * fine box, out[8..15] fluid cells of the physical fine block, each
 * (max |u|^2, max |rho - 1|, sum (rho - 1), sum jx, sum jy, sum jz, cells,
 * non-finite cells) in the level's lattice units. */
int ak_refined_integrals(ak_refined *r, double *out);
/* ak_refined_step without loads, timed with CUDA events on the case's stream:
 * ms[0] whole interval, ms[1] coarse collide, ms[2] coarse stream, ms[3] fine
 * collides, ms[4] fine streams, ms[5] the rest (interface transfers, face
 * fluxes, boundaries, walls), milliseconds summed over the steps.  When the
 * fine box lies three coarse cells inside the lattice the coarse streaming is
 * fused with the next step's collision: ms[1] then covers the collision of
 * the transfer block (the box and three cells around it) alone and ms[2] the
 * fused pass.  No counterpart in the reference; it exists for measurement. */
int ak_refined_step_timed(ak_refined *r, int32_t nsteps, double *ms);
/* RefinedSolver.states() (interface.py:354-358): the pre-collision
 * populations of both levels, coarse (nx, ny, nz, 27) and the padded fine
 * block (2 bx + 4, 2 by + 4, 2 bz, 27), either output may be NULL.  Where the
 * engine keeps the coarse level post-collision (the streaming fused with the
 * next collision outside the box and three cells around it) the
 * pre-collision state is rebuilt by pulling from the copy the last step read;
 * after ak_set_pdf on the coarse level it is known again after the next
 * step (AK_ERR_INVALID until then). */
int ak_refined_states(ak_refined *r, double *coarse, double *fine);
/* One interface kernel of the two-level step, run alone on the levels'
 * current population copies, so that each can be compared with the
 * reference's transfer algebra in isolation:
 *   op 0  donors: moments of the coarse donor block (interface.py:257-263,
 *         refinement.py:148-175), the 5-point prolongation (refinement.py:
 *         78-105), the coarse -> fine stress rescale and the fine padding
 *         band's populations (refinement.py:177-213), coarse-time fraction 0
 *   op 1  restriction of the fine block onto the covered coarse cells
 *         (refined_solver.py:183-188, refinement.py:108-114, 245-254)
 *   op 2  face fluxes (interface.py:44-104) of the coarse copy and of the
 *         fine copy: out[0, n/2) the coarse registers, out[n/2, n) the fine
 *         ones (2 x 2 fine entries summed per coarse entry), n in *n_out;
 *         out = NULL only reports n
 *   op 3  reflux (interface.py:285-295) of the coarse copy from the
 *         registers op 2 left.
 * A failed positivity or Mach check returns AK_ERR_NONFINITE.  No
 * counterpart in the reference; it exists for unit tests. */
int ak_refined_probe(ak_refined *r, int32_t op, double *out, int64_t *n_out);
/* The level's lattice (0 coarse, 1 fine block) for ak_get_pdf / ak_macros /
 * ak_get_wall_links; owned by the refined case.  When the fine box lies three
 * coarse cells inside the lattice, the coarse level holds post-collision
 * populations outside the box and three cells around it (the coarse
 * streaming is fused with the next step's collision); mass and momentum, and
 * so ak_macros, are those of the pre-collision state. */
ak_case *ak_refined_level(ak_refined *r, int32_t level);

/* ---- batches of independent uniform cases --------------------------------
 * No reference counterpart: the reference runs one case per process.  A batch
 * borrows n uniform cases with the characteristic farfield or the legacy
 * outer boundary (one storage form, one device) and advances them together:
 * per step one launch each for the farfield ring macros and links, the UBB
 * cells and outflow links, and the Bouzidi walls of every case, and one
 * stream-collide launch over a packed table of all cases' blocks (one block
 * per table entry in the FP32 and FP16 forms, a persistent grid looping over
 * the table in the FP64 and df64 forms), replayed from CUDA graphs.  A case computes the same bits alone (ak_step)
 * and in a batch.  While a case belongs to a batch, step it only through the
 * batch; its state can be read with the per-case calls. */
typedef struct ak_batch ak_batch;
int ak_batch_create(ak_case *const *cases, int32_t n, ak_batch **out);
int ak_batch_destroy(ak_batch *b);
/* nsteps steps of every case; with loads non-null, loads[case * 40 + element
 * * 5 + k] = that case's per-element (Fx, Fy, Fz, Mz, mass) of the last step,
 * as ak_step returns them. */
int ak_batch_step(ak_batch *b, int32_t nsteps, double *loads);
/* Times the stream-collide launch for every block width (64, 128, 256),
 * persistent grid size (1, 2, 4, ... CTAs per SM up to the occupancy limit;
 * FP64 and df64 forms) and table order (case-major, interleaved), trials
 * launches each, and keeps
 * the fastest.  The cases' state is unchanged.  report[5] = chosen width,
 * CTAs per SM, order, its ms per launch, the previous schedule's ms. */
int ak_batch_tune(ak_batch *b, int32_t trials, double *report);
int64_t ak_batch_launches(const ak_batch *b);
int64_t ak_batch_steps_done(const ak_batch *b);
/* The batch's CUDA stream (cudaStream_t), for callers that time it. */
void *ak_batch_stream(const ak_batch *b);

/* Message of the last failure on this thread ("" if none). */
const char *ak_last_error(void);
/* Library build identification, e.g. "aerokinetic_gb300 sm_103a". */
const char *ak_version(void);
/* Fused multiply-add throughput of the current device in TFLOP/s (two FLOPs
 * per FMA), precision 0 = FP64, 1 = FP32, 2 = packed FP32x2 (two FMAs per
 * instruction and lane): eight dependent FMA chains per
 * thread over 8 blocks of 256 threads per SM, best of three timed launches
 * (CUDA events).  The ceiling of the FP64-bound plain collision.  No
 * counterpart in the reference; it exists for measurement. */
int ak_fma_peak(int32_t precision, double *tflops);
/* Algorithmic floating-point operations of one cell's collision in the form
 * the storage type uses (AK_STORAGE_F64 / F16: the chimera form, F32: the
 * deviation form), counted by evaluating the same collision template on a
 * counting number type: counts[0] additions and subtractions, counts[1]
 * multiplications, counts[2] divisions, counts[3] their sum (a fused
 * multiply-add of the compiled kernel counts as one multiplication and one
 * addition).  No counterpart in the reference; it exists for measurement. */
int ak_collision_flops(int32_t storage, double *counts);

#ifdef __cplusplus
}
#endif
#endif
