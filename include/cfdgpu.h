/*
 * cfdgpu.h — C ABI of the GB300 pressure-projection engine for CFD-craft.
 *
 * The engine replaces the projection step of crates/cfd-craft: the divergence
 * right-hand side, the IC(0)- or multigrid-preconditioned CG solve and the
 * velocity correction. The caller keeps its grid (crates/cfd-craft/src/grid.rs)
 * and hands the engine the grid's products once; the engine keeps the topology,
 * the IC(0) factor and the multigrid hierarchy resident in device memory.
 *
 * Conventions
 *  - Every pointer argument is caller-owned HOST memory, only read during the call
 *    (copied in/out), except parameters named d_* (and those of functions whose name
 *    ends in _device): those are DEVICE memory, used in stream order on the grid's,
 *    batch's or server's stream.
 *  - Cell index (k*ny + j)*nx + i, x fastest (grid.rs:218-220). Face arrays hold
 *    the x-faces, then the y-faces, then the z-faces, each x fastest over its
 *    face dimensions (grid.rs:341-429).
 *  - Return codes map 1:1 to the reference's error strings (see CFDG_*). On any
 *    nonzero return, the caller's u, p and x are unchanged (pressure.rs:468).
 *  - cfdg_last_error() gives the full message ("CFD-E033: ...") of the last
 *    failing call on the calling thread.
 *  - Two threads may use two different grids at once. One grid is used by one
 *    thread at a time (its calls are serialised by an internal lock).
 *  - No CPU fallback: without a usable CUDA device every call that computes
 *    returns CFDG_ERR_CUDA.
 */
#ifndef CFDGPU_H
#define CFDGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Return codes. */
#define CFDG_OK 0
#define CFDG_E031 31            /* incompatible flux in a closed fluid component (pressure.rs:359) */
#define CFDG_E032 32            /* pressure CG lost positive definiteness (pressure.rs:395) */
#define CFDG_E033 33            /* pressure iteration limit (pressure.rs:435) */
#define CFDG_E034 34            /* multigrid topology or weights (multigrid.rs:152,193) */
#define CFDG_E035 35            /* coarse Cholesky / aggregation failure (multigrid.rs:490, masked.rs:42,235) */
#define CFDG_E036 36            /* line Cholesky (multigrid/line.rs:130) */
#define CFDG_CANCELLED 100      /* Control::check() == "cancelled" (solver.rs:122-140) */
#define CFDG_WALL_TIME 101      /* Control::check() == "wall_time_limit" */
#define CFDG_ERR_CUDA 200       /* CUDA error or no usable device */
#define CFDG_ERR_ADMISSION 201  /* the grid does not fit the context's HBM budget */
#define CFDG_ERR_TIMEOUT 202    /* a bounded device wait gave up */
#define CFDG_ERR_INVALID 203    /* invalid argument or inconsistent grid description */
#define CFDG_ERR_UNSUPPORTED 204/* a configuration this engine does not implement */
#define CFDG_PENDING 3          /* cfdg_poll_result: the ticket is not finished yet */

/* Face kinds (grid.rs:60-81). */
#define CFDG_FACE_INTERIOR 0
#define CFDG_FACE_WALL 1
#define CFDG_FACE_SLIP 2
#define CFDG_FACE_INLET 3
#define CFDG_FACE_OUTLET 4
#define CFDG_FACE_BLOCKED 5

/* Preconditioners (case.rs:860-879) and arithmetic forms. */
#define CFDG_PRECOND_IC0 0
#define CFDG_PRECOND_MULTIGRID 1
#define CFDG_PRECISION_PLAIN 0 /* FP64 throughout: the parity form */
#define CFDG_PRECISION_MIXED 1 /* FP32 inner solve, FP64 dots, true residual and refinement */

typedef struct cfdg_context cfdg_context;
typedef struct cfdg_grid cfdg_grid;

/* The grid's products, as crates/cfd-craft/src/grid.rs holds them (Grid, grid.rs:114-162). */
typedef struct {
  int32_t n[3];                 /* cells per axis */
  double dx[3];                 /* Grid::dx */
  double volume;                /* Grid::volume */
  int32_t periodic[3];          /* 1 when the axis wraps (no duplicate end face) */
  int64_t n_faces;              /* Grid::faces.len() */
  const uint8_t *fluid;         /* [N] 1 fluid, 0 solid */
  const uint8_t *face_kind;     /* [F] CFDG_FACE_* */
  const int64_t *face_lo;       /* [F] fluid cell below the face, -1 for none (Face::lo) */
  const int64_t *face_hi;       /* [F] fluid cell above the face, -1 for none (Face::hi) */
  const double *face_area;      /* [F] Face::area, current coefficients */
  const double *face_distance;  /* [F] Face::distance */
  const int32_t *component;     /* [N] fluid component per cell, -1 for solid (Grid::component) */
  int32_t n_components;         /* Grid::components.len() */
  const uint8_t *anchored;      /* [n_components] 1 when the component touches an outlet */
  int32_t preconditioner;       /* CFDG_PRECOND_* (numerics.pressure_preconditioner) */
  int32_t precision;            /* CFDG_PRECISION_* */
} cfdg_grid_desc;

/* LinearInfo (pressure.rs:30-36) plus the phase-profile work counters
 * (profiling.rs:101-138, multigrid.rs:76-114). */
typedef struct {
  uint64_t iterations;          /* PCG iterations; 0 for a zero right-hand side */
  double relative_residual;     /* recomputed residual relative to |b_compatible| */
  uint64_t work_units;
  uint64_t operator_applications;
  uint64_t preconditioner_applications;
  uint64_t true_residual_checks;
  uint64_t hierarchy_builds;
  uint64_t hierarchy_levels;
  uint64_t hierarchy_cells;
  uint64_t hierarchy_nonzeros;
  uint64_t cycles;
  uint64_t smoothing_cell_updates;
  uint64_t residual_cell_updates;
  uint64_t restriction_cell_updates;
  uint64_t prolongation_cell_updates;
  uint64_t coarse_solves;
  uint64_t refinement_steps;    /* outer FP64 defect-correction steps (mixed form); 0 plain */
  double device_seconds;        /* device time of the solve, from CUDA events */
  uint64_t graph_launches;      /* captured iteration chunks replayed by the solve */
  double loop_seconds;          /* device time of the iteration loop alone */
  /* MultigridWork (multigrid.rs:89,103-114): */
  uint64_t hierarchy_bytes;     /* device bytes the hierarchy retains (this engine's storage) */
  uint64_t block_smoothing_cell_updates; /* cell updates of line/plane block sweeps */
  uint64_t block_solves;        /* exact line or plane block solves */
  uint64_t block_level_cell_visits; /* cells of the block-smoothed levels per visit */
  /* The setup spans (profiling.rs Phase::PressureFactorSetup / PressureMultigridSetup,
   * pressure.rs:60-63,79-83): host wall seconds of building the IC(0) factor, and of
   * (re)building the multigrid hierarchy with its upload (plus, in the mixed form, the
   * first build of its FP32 state), inside this call; 0 when the cached one was used. */
  double factor_setup_seconds;
  double multigrid_setup_seconds;
} cfdg_info;

/* Control::check (solver.rs:122-140): 0 continue, 1 "cancelled", 2 "wall_time_limit".
 * Polled before PCG iterations 0, 8, 16, ... like pressure.rs:387-389, and before
 * a multigrid setup (pressure.rs:69). */
typedef int (*cfdg_poll_fn)(void *ctx);

/* ------------------------------------------------------------------ lifetime */

/* Creates a context on CUDA device `device`. hbm_budget_bytes bounds the device
 * memory of all grids opened on it (0 = 90 % of the free memory at creation).
 * Replaces: nothing in the reference (the reference has no device). */
int cfdg_context_create(int device, uint64_t hbm_budget_bytes, cfdg_context **out);
void cfdg_context_destroy(cfdg_context *ctx);

/* Uploads a grid's topology and face coefficients. Replaces the per-grid caches
 * Grid::pressure_factor (grid.rs:151) and Grid::pressure_multigrid (grid.rs:155):
 * the IC(0) factor is built by the first IC(0) solve and never rebuilt (pressure.rs:62-65);
 * the hierarchy is rebuilt when the signature changes (pressure.rs:67-95). */
int cfdg_grid_open(cfdg_context *ctx, const cfdg_grid_desc *desc, cfdg_grid **out);
void cfdg_grid_close(cfdg_grid *grid);

/* Replaces the public face coefficients (callers may change Grid::faces[*].area
 * and .distance, pressure.rs:244). The operator and the true residual use them on
 * the next solve; the IC(0) factor is kept (pressure.rs:714-743); a changed weight
 * rebuilds the multigrid hierarchy before the next solve (multigrid.rs:173-222). */
int cfdg_grid_update_faces(cfdg_grid *grid, const double *face_area, const double *face_distance);

/* Switches the preconditioner or the arithmetic form of an open grid. */
int cfdg_grid_configure(cfdg_grid *grid, int32_t preconditioner, int32_t precision);
/* ------------------------------------------------------------------ laminar time stepping
 * The flow terms of the case that the projection does not read (case.rs Flow::Laminar,
 * boundaries, domain size), for cfdg_step_device. Open, wall and slip boundaries. */
typedef struct {
  int32_t boundary[3];     /* per axis: 1 open, 2 wall, 3 slip (case.rs Boundary) */
  double size_m[3];        /* domain size */
  double velocity[3];      /* initial_velocity_m_s: the inflow (Flow::vector) */
  double viscosity;        /* viscosity_m2_s */
  double acceleration[3];  /* acceleration_m_s2 */
} cfdg_flow_desc;
int cfdg_grid_set_flow(cfdg_grid *grid, const cfdg_flow_desc *flow);
/* One SSPRK2 step of laminar flow with a projection per stage, in place on device arrays
 * d_u (F) and d_p (N) (solver.rs:879-960 with flow_euler solver.rs:671-732; the momentum
 * right-hand side flow.rs:426-525 with donor-cell advection). Each stage projects in the
 * grid's precision (plain: bit-identical to the reference algorithm). On any error u and
 * p are unchanged. info: the second projection's, with iterations and work summed. */
int cfdg_step_device(cfdg_grid *grid, double *d_u, double *d_p, double dt, double tol, uint64_t max_iter,
                     cfdg_poll_fn poll, void *poll_ctx, cfdg_info *info);
/* One SSPRK2 step of a constituent's concentration d_c (N, kg/m3) in place on the face
 * velocities d_u (F), with cell diffusivities d_diff (N, m2/s: the constituent's plus
 * nu_t / Sc) and source densities d_source (N, kg/m3/s): advance_scalar
 * (solver.rs:808-855) with the grid's advection scheme (linear upwind unless
 * cfdg_grid_set_advection selects MUSCL; transport.rs:651-699) and zero inflow
 * concentration, bit-identical to it; the budgets are not kept (cfdg_scalar_step_budget
 * keeps them). Non-periodic grids. */
int cfdg_scalar_step_device(cfdg_grid *grid, const double *d_u, double *d_c, const double *d_diff,
                            const double *d_source, double dt);
/* The same step, and its mass budget (solver.rs:851-853): d_budget (device, three doubles:
 * emitted, inflow, outflow in kg) grows by dt/2 times the sum of the two stages' rates,
 * each the one rhs_into returns (transport.rs:651-699: source sum times the cell volume,
 * and the positive and negative parts of the outward flux over the domain-boundary faces).
 * The concentration gets the same bits as cfdg_scalar_step_device; the rates are summed
 * in a fixed order of their own, within rounding of the reference's sequential sums. */
int cfdg_scalar_step_budget(cfdg_grid *grid, const double *d_u, double *d_c, const double *d_diff,
                            const double *d_source, double dt, double *d_budget);
/* The current rates of d_c (kg/s) into the host array rates: emitted, inflow, outflow, as
 * rhs_into returns them (the summary's source and boundary rates, solver.rs ScalarEvidence). */
int cfdg_scalar_rates(cfdg_grid *grid, const double *d_u, const double *d_c, const double *d_diff,
                      const double *d_source, double *rates);
/* The advection scheme of the grid's scalar steps and rates (Advection, transport.rs:
 * 502-526, 670-694): 0 linear upwind (the default), 1 MUSCL, whose donor value is the
 * upwind cell's value plus or minus half its monotonized-central limited slope along the
 * face's axis (neighbours through interior faces only). Either is bit-identical to the
 * reference's rhs_into. Other values: CFDG_ERR_INVALID. */
int cfdg_grid_set_advection(cfdg_grid *grid, int32_t muscl);
/* Receptors of a grid for cfdg_receptors_sample: n receptors' normalised weights as
 * receptor_weights (transport.rs:374-436) returns them, in CSR form: receptor r holds
 * cells[offsets[r] .. offsets[r+1]) with weights[...] in that order (host arrays, copied).
 * Cells must lie in the grid; an empty receptor is CFDG_ERR_INVALID (the reference's E042
 * is raised where the weights are made). Replaces the receptors set before. */
int cfdg_receptors_set(cfdg_grid *grid, int32_t n, const int64_t *offsets, const int64_t *cells,
                       const double *weights);
/* The receptor values of the concentration d_c (device, N doubles) into d_out (device, n
 * doubles), on the grid's stream: each the sum of c[cell] w in weight order, as the monitor
 * row of solver.rs:1024-1041 computes it, bit-identical. */
int cfdg_receptors_sample(cfdg_grid *grid, const double *d_c, double *d_out);
/* Diagnostic: one stage's velocity before its projection, out = u + dt (R(u) - grad p) with
 * the fixed face values, on host arrays (F, N, F doubles). No reference counterpart. */
int cfdg_debug_momentum_update(cfdg_grid *grid, const double *u, const double *p, double dt, double *out);

/* Mixed form: Gauss-Seidel sweeps before and after the coarse correction of the V-cycle,
 * on level 0 and on the coarse levels (1..4 each; default 2 and 2, the reference's
 * V(2,2)). Batches and servers created afterwards take the counts from their grids (all
 * grids of one batch must agree), so a grid gives the same result alone and in a batch.
 * The bench's autotuner picks them per case mix. No reference counterpart. */
int cfdg_grid_set_cycle(cfdg_grid *grid, int32_t nu_fine, int32_t nu_coarse);
/* Mixed form: tile shape of the level-0 red-black half sweeps, which the tensor memory
 * accelerator stages through shared memory on grids with uniform weights and ceil(nx/2) a
 * multiple of 8: rows per stage (8, 16 or 32; the y halo is two rows per stage) and stages
 * in flight per block (2..8; fewer when they do not fit the shared memory). 0 and 0 (the
 * default) choose from the row length: two stages of 32 rows when two blocks of them fit an
 * SM's shared memory, else of 16 or 8 rows.
 * Batches and servers created afterwards take it from their grids (all grids of one batch
 * must agree); the results do not depend on it, bit for bit. The bench's autotuner picks it
 * per case mix. No reference counterpart. */
int cfdg_grid_set_sweep_tile(cfdg_grid *grid, int32_t rows, int32_t stages);
/* Mixed form on aggregation (masked) hierarchies: the coarse corrections of the V-cycle are
 * scaled by alpha, 0 < alpha < 2 (default 1.8; 1 is the reference's cycle). The piecewise-
 * constant prolongation under-corrects smooth errors; on the 52-case wind-direction mix
 * with V(2,2) 1.85 took the iterations to 1e-8 from 33 to 8. The stopping test is the FP64 true
 * residual, so the result meets the same tolerance. Batches and servers created afterwards
 * take it; grids with linear interpolation (no solid cells) are not scaled. */
int cfdg_grid_set_coarse_scale(cfdg_grid *grid, double alpha);
/* Mixed form: the first coarse level of an aggregation hierarchy laid out as the grid of
 * 2x2x2 bins (bins = 1, the default) where every bin holds at most one aggregate, the
 * level has no closed groups and the weights are uniform; the level-0 residual is then
 * formed inside the restriction and a cell's parent is its bin. bins = 0 keeps the
 * aggregates in colour order with index lists. Both give the same bits; a batch or server
 * takes the layout from its grids. No reference counterpart. */
int cfdg_grid_set_coarse_layout(cfdg_grid *grid, int32_t bins);

/* ------------------------------------------------------------------ the projection */

/* pressure::project (pressure.rs:469-502): solves A phi = -div(u)/dt, subtracts
 * dt*grad(phi) from the interior and outlet faces of u[F], adds phi to p[N] and
 * re-centres p's gauge. Called from solver.rs:721, :767 and :1437. */
int cfdg_project(cfdg_grid *grid, double *u, double *p, double dt, double tol, uint64_t max_iter,
                 cfdg_poll_fn poll, void *poll_ctx, cfdg_info *info);

/* pressure::solve_scaled (pressure.rs:342-436): x[N] solves A x = b with the
 * compatibility check against roundoff_scale[N] (NULL: |b|), PCG with the grid's
 * preconditioner and the true-residual gate. pressure::solve (pressure.rs:329) is
 * roundoff_scale == NULL. */
int cfdg_solve_scaled(cfdg_grid *grid, const double *b, const double *roundoff_scale, double tol,
                      uint64_t max_iter, cfdg_poll_fn poll, void *poll_ctx, double *x, cfdg_info *info);

/* pressure::apply (pressure.rs:293-312): y = A x from the current faces, bitwise equal
 * to the reference's face-order accumulation. */
int cfdg_apply(cfdg_grid *grid, const double *x, double *y);

/* pressure::center_nullspaces (pressure.rs:316-325). */
int cfdg_center_nullspaces(cfdg_grid *grid, double *x);

/* pressure::multigrid_stats (pressure.rs:100-106) as JSON, MultigridStats
 * (multigrid.rs:55-72): {"level_cells":[...],"level_dimensions":[[nx,ny,nz],...],
 * "level_nonzeros":[...],"allocated_bytes":B,"block_smoothers":[{"level","axes",
 * "block_unknowns","block_count","half_bandwidth","allocated_bytes"},...]}, the empty
 * level_dimensions (masked hierarchies) and block_smoothers (point smoothing) omitted as
 * the reference's serialisation does; the byte counts are this engine's device storage. Returns
 * CFDG_PENDING when no hierarchy was built yet. Safe to call from a poll callback. */
int cfdg_multigrid_stats_json(cfdg_grid *grid, char *buf, size_t cap);

/* Last error message of the calling thread ("" when none). */
const char *cfdg_last_error(void);

/* ------------------------------------------------------------------ device-resident forms */

/* cfdg_project on device pointers (u: F doubles, p: N doubles), on the grid's
 * stream. u and p are updated only on success. */
int cfdg_project_device(cfdg_grid *grid, double *d_u, double *d_p, double dt, double tol,
                        uint64_t max_iter, cfdg_poll_fn poll, void *poll_ctx, cfdg_info *info);

/* ------------------------------------------------------------------ batched mixed-precision form
 * The projection of several grids at once in the mixed form: FP32 inner PCG with an
 * FP32 V-cycle (red-black / multicolour Gauss-Seidel on the reference hierarchy), FP64
 * dot products, alpha/beta, true residual, outer defect correction and coarsest
 * solve. Each case stops when its FP64 relative residual |b_c - A x|/|b_c| <= tol.
 * Every grid must be open on the batch's context, non-periodic, and its multigrid
 * hierarchy is built (or reused) at creation. A batch keeps its own FP32 state;
 * the grids stay owned by the caller and must outlive the batch. */
typedef struct cfdg_batch cfdg_batch;
int cfdg_batch_create(cfdg_context *ctx, cfdg_grid *const *grids, int32_t n, cfdg_batch **out);
void cfdg_batch_destroy(cfdg_batch *batch);
int cfdg_batch_set_stream(cfdg_batch *batch, void *stream);
int cfdg_batch_size(const cfdg_batch *batch);
/* pressure::project for every case i (host u[i], p[i]); codes[i] is case i's return
 * code and a failed case keeps its u[i], p[i]. Returns nonzero only for a failure of
 * the whole call (CUDA error, cancellation). */
int cfdg_batch_project(cfdg_batch *batch, double *const *u, double *const *p, const double *dt, double tol,
                       uint64_t max_iter, cfdg_poll_fn poll, void *poll_ctx, cfdg_info *infos, int32_t *codes);
/* Times one unit of the batch's work `reps` times with CUDA events on the batch's
 * stream, every case in its inner-iteration state: which = 0 one red-black half sweep
 * over all fine levels, 1 the FP32 operator, 2 all coarse levels (one cooperative launch), 3 one
 * V-cycle, 4 the half sweep of 0 with the unstaged register kernel, 5 the FP64 true
 * residual of every case, 6 the FP64 right-hand side of every case (only after a
 * host-buffer cfdg_batch_project, whose inputs the batch keeps), 7 the level-0 residual
 * with its restriction to level 1, 8 the prolongation of the level-1 correction to level
 * 0, 9 the inner update (e, r and |r|^2), 10 r.z, 11 p = z + beta p. Reports the mean duration
 * and the unit's algorithmic bytes (0 when not stated). Diagnostic; no reference
 * counterpart. */
int cfdg_batch_time_kernel(cfdg_batch *batch, int32_t which, int32_t reps, double *ms_per_launch,
                           double *algorithmic_bytes);
/* Per case and coarse level of the batch's FP32 hierarchies, as JSON: rows, nonzeros,
 * smoother colours, ELL entries (with padding), closed groups and terminal blocks; and
 * whether level 1 is laid out as the bin grid ("level1_bins", per case) and swept through
 * computed bin-stencil columns ("level1_stencil"; per level "bin_stencil"), and
 * whether the level-0 half sweeps run staged through the tensor memory accelerator
 * ("staged_sweeps": every case with uniform weights and ceil(nx/2) a multiple of 8). Writes
 * at most cap bytes (NUL-terminated) and returns the length the full text needs, or a
 * negative error code. Diagnostic; no reference counterpart. */
int64_t cfdg_batch_stats_json(cfdg_batch *batch, char *buf, int64_t cap);
/* Copies case c's FP64 right-hand side b = -div(u)/dt and its round-off terms (0 unless
 * the grid has closed components) of the batch's last projection to host arrays of N
 * doubles. Diagnostic (parity of the mixed form's right-hand side); no reference counterpart. */
int cfdg_batch_debug_rhs(cfdg_batch *batch, int32_t c, double *b, double *terms);
/* Counts the numerators x, of n generated from seed (mode 0 random over 2^+-900, 1 next to
 * y times a double, 2 next to y times a midpoint), whose quotient x / y by the engine's
 * division from a precomputed reciprocal differs in any bit from the correctly rounded
 * division. Diagnostic; no reference counterpart. */
int cfdg_debug_div_check(double y, uint64_t seed, int64_t n, int32_t mode, uint64_t *mismatches);
/* The same on device arrays d_u[i] (F_i doubles) and d_p[i] (N_i doubles). */
int cfdg_batch_project_device(cfdg_batch *batch, double *const *d_u, double *const *d_p, const double *dt,
                              double tol, uint64_t max_iter, cfdg_poll_fn poll, void *poll_ctx, cfdg_info *infos,
                              int32_t *codes);

/* ------------------------------------------------------------------ serving (continuous batching)
 * A server keeps `n` resident grids (their topology, hierarchy and FP32 state stay in HBM
 * across requests; cfdg_grid_open already refused grids beyond the context's HBM budget)
 * and runs projection requests on them in the mixed form. cfdg_server_progress() is one
 * scheduling round: it finishes the requests whose cases converged in the previous round
 * (face correction, p update, result recorded), admits queued requests into free slots
 * (at most max_active running at once; one request per grid at a time, in arrival order),
 * and replays one chunk of the batched iteration over the running cases, so requests that
 * arrive while others are on the GPU join them at the next chunk. Results are
 * bit-identical to the same request solved alone. No reference counterpart: the
 * reference runs one case per process. */
typedef struct cfdg_server cfdg_server;
int cfdg_server_create(cfdg_context *ctx, cfdg_grid *const *grids, int32_t n, int32_t max_active,
                       cfdg_server **out);
void cfdg_server_destroy(cfdg_server *server);
int cfdg_server_set_stream(cfdg_server *server, void *stream);
/* Queues pressure::project on grid `grid` for device arrays d_u (F doubles), d_p (N doubles),
 * which must stay valid until the ticket's result is read. */
/* Iterations per graph chunk (1..64, default 4): requests join and leave the running set
 * at chunk boundaries, so shorter chunks lower latency at more host rounds. */
int cfdg_server_set_chunk(cfdg_server *server, int32_t iterations);
int cfdg_server_submit(cfdg_server *server, int32_t grid, double *d_u, double *d_p, double dt, double tol,
                       uint64_t max_iter, uint64_t *ticket);
/* The same request on host buffers: the engine copies u (F doubles) and p (N doubles) to
 * one of two device slots of the grid on a copy stream of its own (the request starts once
 * the copy is done), and after the request copies the projected fields, or on failure the
 * unchanged inputs, into u_out and p_out on another copy stream; cfdg_server_result reports
 * the ticket done only when those copies have completed. All four buffers must stay valid
 * until then; page-locked host memory lets the copies overlap the solves. A grid's next
 * input copy waits until the results of the request that last used its slot have been
 * copied out; a third request of a grid while two are unfinished is CFDG_ERR_INVALID. The
 * reference-facing form of serving: the caller's fields stay in host memory. */
int cfdg_server_submit_host(cfdg_server *server, int32_t grid, const double *u, const double *p, double *u_out,
                            double *p_out, double dt, double tol, uint64_t max_iter, uint64_t *ticket);
int cfdg_server_progress(cfdg_server *server, int32_t *finished);
/* 0 and the result (consumed) when the ticket finished, CFDG_PENDING otherwise. */
int cfdg_server_result(cfdg_server *server, uint64_t ticket, cfdg_info *info, int32_t *code);
/* Requests queued or running. */
int cfdg_server_pending(cfdg_server *server);
/* Counters of the server since its creation, as JSON: progress rounds, graph chunks
 * launched and their device time (CUDA events around each launch), host time spent in
 * cfdg_server_progress (it includes waiting for the previous chunk) and the part of it
 * after that wait, the device time from the end of a chunk to the start of the next one
 * launched in the following round (epilogues, prologues and the device waiting on the
 * host) with the number of such pairs, requests finished and admitted. Same buffer
 * convention as cfdg_batch_stats_json. No reference counterpart. */
int64_t cfdg_server_stats_json(cfdg_server *server, char *buf, int64_t cap);

/* Device memory the grid holds, in bytes (admission accounting). */
uint64_t cfdg_grid_device_bytes(const cfdg_grid *grid);

/* No reference counterpart: an addition for callers that cannot allocate device memory.
 * Writes |A x - b| / |b| for device vectors x[N], b[N] of an open grid to d_out[0], on
 * `stream` (NULL: the grid's stream), without waiting for it; 0 when |b| < 1e-24, as
 * the solve reports for a zero right-hand side (pressure.rs:372-375). b is used as
 * given, not centred: the value equals the relative residual of the solve's acceptance
 * gate (pressure.rs:403-415), which uses the centred b, on grids whose fluid components
 * all touch an outlet, or for a b whose closed components already have zero mean. Some callers cannot call
 * cudaMalloc: a host that has handed the whole HBM budget to resident serving state, a
 * step that must not block on the implicit device synchronisation an allocation can
 * cause, or code running where an allocation failure cannot be handled. This entry
 * point allocates nothing: its per-block partial sums live in a static device array of
 * 128 KiB + 256 B that every GPU loading the library holds until exit, which limits it
 * to grids of at most 16,777,216 cells (larger grids return CFDG_ERR_INVALID). The
 * first call on a device looks up that array's address, so make it before any stream
 * capture. All calls share the array: calls that overlap on the GPU race. */
int cfdg_residual_norm_noalloc(cfdg_grid *grid, const double *d_x, const double *d_b, double *d_out, void *stream);

/* Enqueues the grid's work on `stream` (a cudaStream_t; NULL: the grid's own stream),
 * so a caller can order it with its own kernels and time it with its own events. */
int cfdg_grid_set_stream(cfdg_grid *grid, void *stream);

/* ------------------------------------------------------------------ diagnostic entry points
 * Pieces of the projection exposed for parity tests; no reference counterpart is
 * replaced by them. */

/* z = M^-1 r for the grid's preconditioner (pressure.rs:43-53): IC(0) Factor::apply
 * (pressure.rs:223-241) or one V-cycle (multigrid.rs:656-665, masked.rs:292-302). */
int cfdg_debug_precondition(cfdg_grid *grid, const double *r, double *z);

/* projection_rhs (pressure.rs:440-459): b[N], terms[N] from u[F]. */
int cfdg_debug_projection_rhs(cfdg_grid *grid, const double *u, double dt, double *b, double *terms);

/* Test hook of the bounded device waits: from the next solve on, wavefront tile
 * hold_tile (-1: none) of the grid's structured sweeps never publishes its progress, and
 * every wait gives up after spin_limit polls (1 .. the default of about a second). The
 * tiles that wait for the held tile give up, raise the sweep's abort flag so the others
 * return too, and the call reports CFDG_ERR_TIMEOUT with u, p and x unchanged; the
 * context stays usable. hold_tile = -1 with the default limit restores normal sweeps.
 * CFDG_ERR_UNSUPPORTED on grids with a periodic axis (no wavefront sweeps). */
int cfdg_debug_wave_stall(cfdg_grid *grid, int32_t hold_tile, int64_t spin_limit);

/* Number of kernels this library has enqueued since it was loaded (a CUDA-graph
 * launch counts its kernel nodes). */
uint64_t cfdg_launch_count(void);

/* Times one unit of work `reps` times on the grid's stream with CUDA events:
 * which = 0 the operator y = A x, 1 one fine-level Gauss-Seidel sweep, 2 one IC(0)
 * application (forward + backward), 3 one V-cycle. Reports the mean duration and the
 * unit's algorithmic bytes (each logical array read or written once). */
int cfdg_debug_time_kernel(cfdg_grid *grid, int32_t which, int32_t reps, double *ms_per_launch,
                           double *algorithmic_bytes);

#ifdef __cplusplus
}
#endif

#endif /* CFDGPU_H */
