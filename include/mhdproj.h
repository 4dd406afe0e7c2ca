/*
 * mhdproj.h -- C ABI of the GB300 MAC pressure projection.
 *
 * Drop-in replacement for the projection of sdfgeoff/mhd-simulator's fluid
 * solver: FluidState::project(warm_start) -> Result<(u32, f32), String>
 * (src/fluid/mod.rs:1015-1115) together with the coefficient cache it builds
 * (pressure_coefficients, src/fluid/solver.wgsl:93-103), the gauge selection
 * (configure_pressure_projection and anchors, src/fluid/mod.rs:978-1002 and
 * :1447-1493) and the pressure written by `fields` (p = rho_l * phi / dt,
 * src/fluid/solver.wgsl:269-270).  The reference's method is private Rust on
 * wgpu buffers; this header is the FFI boundary a Rust crate would bind
 * instead.
 *
 * Conventions
 *  - Cells are indexed x-fastest: i = x + nx*(y + ny*z) (src/simulation.rs:319-323).
 *  - Face velocities are three SoA arrays of FP32 with shapes
 *      u: (nx+1) x ny x nz,  v: nx x (ny+1) x nz,  w: nx x ny x (nz+1)
 *    (x-fastest).  The reference packs the three components into one vec4
 *    per (n+1)^3 face-cell (solver.wgsl:33-36); only the parity tests convert.
 *    On a periodic axis the last face duplicates face 0: inputs are read at
 *    face 0, outputs are written to both.
 *  - Every pointer argument of the compute entry points is a DEVICE pointer
 *    unless the function name ends in _host.  The context owns its workspace.
 *  - Return value 0 is success; otherwise an mhdproj_status code, with a
 *    message from mhdproj_last_error().  A context is used by one host thread
 *    at a time and issues all work on its own CUDA stream.
 */
#ifndef MHDPROJ_H
#define MHDPROJ_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct mhdproj_ctx mhdproj_ctx;

typedef enum {
    MHDPROJ_OK = 0,
    MHDPROJ_ERR_INVALID = 1,        /* bad argument or configuration */
    MHDPROJ_ERR_CUDA = 2,           /* CUDA runtime error */
    MHDPROJ_ERR_NOT_CONVERGED = 3,  /* "Fluid pressure solve did not converge after N iterations" */
    MHDPROJ_ERR_NONFINITE = 4,      /* "Nonfinite fluid pressure residual" */
    MHDPROJ_ERR_NO_PROGRESS = 5,    /* "Fluid pressure iteration made no progress" */
    MHDPROJ_ERR_STATE = 6,          /* call order (e.g. project before set_coefficients) */
    MHDPROJ_ERR_OUT_OF_MEMORY = 7,  /* workspace does not fit */
    MHDPROJ_ERR_TIMEOUT = 8         /* a bounded host wait on the device expired */
} mhdproj_status;

typedef enum {
    /* Closed domain as in the reference: walls and solid faces are closed,
       the constant null space is fixed by a pinned cell per component or by
       mean-free residuals for a single component (src/fluid/mod.rs:978-1002). */
    MHDPROJ_BOUNDARY_REFERENCE_CLOSED = 0,
    /* Dirichlet p = 0 on the top z-face (a GB300-path extension). */
    MHDPROJ_BOUNDARY_OUTLET_TOP = 1
} mhdproj_boundary;

typedef enum {
    MHDPROJ_PRECISION_FP32 = 0,     /* multigrid level fields in FP32 */
    MHDPROJ_PRECISION_FP16 = 1,     /* multigrid level fields in FP16, FP32 accumulation */
    MHDPROJ_PRECISION_BF16 = 2      /* multigrid level fields in BF16, FP32 accumulation */
} mhdproj_precision;

typedef enum {
    /* The reference algorithm, FP32 throughout: Jacobi-CG below 96^3 cells,
       aggregation-multigrid CG at or above (src/fluid/mod.rs:1030-1096,
       src/fluid/multigrid.rs), with the reference's convergence tests. */
    MHDPROJ_SOLVER_REFERENCE = 0,
    /* The GB300 path: CG preconditioned by a red-black Gauss-Seidel
       aggregation V-cycle with exact coarse solve, FP64 reductions, FP64
       refinement residual on the finest level. */
    MHDPROJ_SOLVER_GB300 = 1
} mhdproj_solver;

typedef enum {
    MHDPROJ_PRECOND_AUTO = -1,      /* reference: by the 96^3 rule; GB300: RBGS multigrid */
    MHDPROJ_PRECOND_JACOBI = 0,
    MHDPROJ_PRECOND_MULTIGRID = 1
} mhdproj_preconditioner;

typedef struct {
    uint32_t nx, ny, nz;
    float h;                /* cell size in metres (GridSi::cell_m) */
    uint32_t periodic;      /* bit a set: axis a is periodic (FluidConfig::periodic) */
    int32_t boundary;       /* mhdproj_boundary */
} mhdproj_grid;

typedef struct {
    int32_t solver;         /* mhdproj_solver */
    int32_t precision;      /* mhdproj_precision (GB300 solver) */
    int32_t preconditioner; /* mhdproj_preconditioner */
    float rel_tol;          /* FluidConfig::relative_tolerance */
    float abs_div_tol;      /* FluidConfig::absolute_divergence_tolerance, 1/s */
    uint32_t max_iterations;/* FluidConfig::max_iterations (all refinement passes) */
    int32_t max_refinements;/* GB300 solver: FP64 refinement passes (>= 1) */
    int32_t two_phase;      /* reference solver: SurfaceConfig::enabled (density from the liquid fraction) */
    int32_t gauge;          /* -1 automatic, 0 pinned cells, 1 mean-free if connected.  Both solvers take the
                               mean-free gauge for one closed component (GB300: the result is zero at the
                               component's first cell; the adjoint needs gauge 0 or an outlet) */
    int32_t compute_divergence; /* fill max/RMS divergence of the projected velocity in the stats */
} mhdproj_options;

typedef struct {
    uint32_t iterations;        /* CG iterations, all passes */
    uint32_t refinements;       /* FP64 residual evaluations after the first (GB300 solver) */
    float relative_residual;    /* reference: sqrt(s[1]/s[2]) of the final check; GB300: FP64 true residual */
    double true_relative_residual; /* ||b - A phi|| / ||b|| evaluated in FP64 */
    double max_divergence;      /* max |div u| over active cells, 1/s (if requested) */
    double rms_divergence;
    float elapsed_ms;           /* device time of the call */
    int32_t meanfree;           /* reference solver: gauge mode used */
    int32_t multigrid;          /* preconditioner used */
    uint32_t levels;            /* multigrid levels */
    uint64_t coarse_cells;      /* cells on levels >= 1 */
} mhdproj_stats;

/* Defaults: GB300 solver, FP16 levels, rel_tol 1e-6, abs floor 0, 20000 iterations. */
void mhdproj_default_options(mhdproj_options *options);

/* FluidState::new's projection set-up (src/fluid/mod.rs:199-330).  Validates the
 * grid and options and allocates the workspace. */
int mhdproj_create(const mhdproj_grid *grid, const mhdproj_options *options, mhdproj_ctx **out);

/* Release the context and its device memory. */
void mhdproj_destroy(mhdproj_ctx *ctx);

/* Message of the last failing call on ctx ("" if none).  ctx may be NULL for
 * errors of mhdproj_create. */
const char *mhdproj_last_error(const mhdproj_ctx *ctx);

/* Issue all work on this cudaStream_t (default: a stream the context owns). */
int mhdproj_set_stream(mhdproj_ctx *ctx, void *stream);

/* Mobility inputs (pressure_coefficients, solver.wgsl:93-103, with mobility()
 * :43-51): liquid fraction per cell (FluidCell.reserved.z) and a solid mask
 * (nonzero = wall cell), plus the liquid and ambient densities.  The fluid
 * mask is every non-solid cell.  The connected components and gauges
 * (anchors(), src/fluid/mod.rs:1447-1493) are recomputed only when the solid
 * mask differs from the previous call, as FluidState::update_cells does. */
int mhdproj_set_coefficients(mhdproj_ctx *ctx, const float *alpha, const uint8_t *solid, float rho_liquid,
                             float rho_air);

/* The thermal phase-fraction drag of mobility() (solver.wgsl:46-50),
 * beta / (1 + dt * rate (1-f)^2 / (f^3 + 1e-3)) with f the smaller phase
 * fraction (FluidCell.reserved.y) of the two cells; phase is a device array of
 * one FP32 per cell, copied by the call.  Pass phase = NULL to disable.  The
 * reference solver applies it at the next mhdproj_set_coefficients; the GB300
 * solver rebuilds its coefficients at once if they are set.  A projection,
 * adjoint or chain with another dt is refused, as the reference rebuilds its
 * coefficients with the step's dt. */
int mhdproj_set_phase_drag(mhdproj_ctx *ctx, const float *phase, float drag_rate, float dt);

/* FluidState::project + correct (src/fluid/mod.rs:1015-1115, solver.wgsl:245-250):
 * project the candidate face velocities u_star onto discretely divergence-free
 * fields.  u_out may alias u_star.  p_out (may be NULL) receives the pressure
 * rho_l * phi / dt per cell (0 in solid cells).  warm_start reuses the previous
 * call's pressure: the reference's pressure_warm/pressure_commit (:164-184) in
 * the reference solver, the previous potential as the initial guess in the
 * GB300 solver.  On failure the outputs are not written. */
int mhdproj_project(mhdproj_ctx *ctx, const float *u_star_x, const float *u_star_y, const float *u_star_z,
                    float *u_out_x, float *u_out_y, float *u_out_z, float *p_out, float dt, int warm_start,
                    mhdproj_stats *stats);

/* The same call on HOST buffers: copies alpha, solid and u_star to the device,
 * sets the coefficients, projects, and copies u_out and p_out back. */
int mhdproj_project_host(mhdproj_ctx *ctx, const float *alpha, const uint8_t *solid, float rho_liquid,
                         float rho_air, const float *u_star_x, const float *u_star_y, const float *u_star_z,
                         float *u_out_x, float *u_out_y, float *u_out_z, float *p_out, float dt, int warm_start,
                         mhdproj_stats *stats);

/* Vector-Jacobian product of the projection with the current coefficients
 * (GB300 solver): given dL/du_out (faces) and dL/dp_out (cells, may be NULL)
 * return dL/du_star.  One adjoint CG solve with the same symmetric operator,
 * then the transposed divergence.  torch.autograd.Function.backward contract. */
int mhdproj_project_vjp(mhdproj_ctx *ctx, const float *grad_u_x, const float *grad_u_y, const float *grad_u_z,
                        const float *grad_p, float dt, float *grad_us_x, float *grad_us_y, float *grad_us_z,
                        mhdproj_stats *stats);

/* Chain u_{k+1} = P(u_k + dt f / rho_face) for `steps` steps from u0 with a
 * fixed face force f (N/m^3); objective J = sum of w^2 over the outlet faces of
 * the final state.  States are checkpointed every `checkpoint_every` steps.
 * The final state is written to u_final (device).  */
int mhdproj_chain_forward(mhdproj_ctx *ctx, const float *u0_x, const float *u0_y, const float *u0_z,
                          const float *f_x, const float *f_y, const float *f_z, float dt, int steps,
                          int checkpoint_every, float *uf_x, float *uf_y, float *uf_z, double *objective,
                          mhdproj_stats *stats);
/* dJ/df of the last mhdproj_chain_forward, by the adjoint chain. */
int mhdproj_chain_backward(mhdproj_ctx *ctx, float *grad_f_x, float *grad_f_y, float *grad_f_z,
                           mhdproj_stats *stats);

/* Objective of the chain for the following mhdproj_chain_forward/backward
 * calls (resets the differentiable chain).  MHDPROJ_CHAIN_FINAL_OUTLET (the
 * default): J = sum of w^2 over the outlet faces of the final state; its
 * adjoint needs no forward state.  MHDPROJ_CHAIN_SUMMED_OUTLET: J = that sum
 * over the states after every step; the backward pass recomputes each
 * checkpoint segment's states from its checkpoint (at most
 * checkpoint_every - 1 forward projections per segment) and keeps a copy of
 * the force from the forward call.  The reference has no adjoint: both
 * objectives are additions of this library. */
enum { MHDPROJ_CHAIN_FINAL_OUTLET = 0, MHDPROJ_CHAIN_SUMMED_OUTLET = 1 };
int mhdproj_chain_set_objective(mhdproj_ctx *ctx, int kind);

/* Probes used by the tests.  y = A x with the solver's operator (reference:
 * apply() of solver.wgsl:78-92 on the cached coefficients, pinned cells as
 * identity rows); z = M r with the solver's preconditioner (reference: the
 * fixed V-cycle of multigrid.wgsl, or r/diag for Jacobi).  x, y, r, z are
 * FP32 device arrays of nx*ny*nz cells. */
int mhdproj_apply_operator(mhdproj_ctx *ctx, const float *x, float *y);
int mhdproj_apply_preconditioner(mhdproj_ctx *ctx, const float *r, float *z);
/* Copy the fine coefficient cache, 4 floats per cell (device pointer):
 * reference solver (beta_x, beta_y, beta_z of the low faces, diagonal) as in
 * velocity[i] of pressure_coefficients; GB300 solver (beta_x, beta_y, beta_z,
 * reaction of outlet and pinned-cell edges). */
int mhdproj_copy_coefficients(mhdproj_ctx *ctx, float *coef4);
/* Copy the last solution potential phi (FP64 device array of nx*ny*nz). */
int mhdproj_copy_potential(mhdproj_ctx *ctx, double *phi);
/* Cell classes after the last topology change (host array of nx*ny*nz):
 * reference solver: the encoded mask of anchors(); GB300 solver: 0 solid,
 * 1 active, 2 pinned gauge cell.  Returns the number of components. */
int mhdproj_copy_topology(mhdproj_ctx *ctx, uint32_t *mask_host, uint32_t *components);

/* Measurement hook: after a projection, time the fine-level kernels of one CG
 * iteration (and the set-up kernels) in isolation, `reps` launches each on the
 * context stream between CUDA events.  For each kernel: its name, the mean
 * device time of one launch, the algorithmic bytes of one launch, and how many
 * times one CG iteration launches it.  Leaves the solver state undefined until
 * the next mhdproj_project. */
typedef struct {
    char name[32];
    float ms;
    double bytes;
    int per_iteration;
} mhdproj_kernel_time;
int mhdproj_profile_kernels(mhdproj_ctx *ctx, int reps, mhdproj_kernel_time *out, int max_out, int *count);

/* Measurement hook, no counterpart in the reference: the number of kernels
 * this context has launched on the GPU since it was created (GB300 solver:
 * coefficient set-up, projections, adjoints and chains; launches inside a
 * replayed CUDA graph count one each, kernels that return early because the
 * solve has converged included). */
int mhdproj_kernel_launches(mhdproj_ctx *ctx, uint64_t *count);

/* Divergence statistics of a face-velocity field that allocate nothing.
 * No counterpart in the reference: it exists for callers that cannot allocate
 * device memory while they run (a time loop that reserved its whole budget at
 * start-up, or a diagnostics hook on another library's stream with no
 * projection context).  Computes out[0] = max |div u| and out[1] = RMS div u
 * (1/s) over the non-solid cells, div u = sum of (u_high - u_low) / h, from
 * device arrays solid (nx*ny*nz) and u, v, w (the face layout above), on the
 * given cudaStream_t (NULL: legacy default stream); returns when the result is
 * on the host.  The reduction scratch is a fixed 96 KiB array in the library's
 * device image (kept by every GPU that loads the library until exit), so an
 * x-y plane may hold at most 4096 tiles of 32x8 cells (nx*ny up to about one
 * million); larger planes, and grids whose face arrays reach 2^31 elements,
 * return MHDPROJ_ERR_INVALID with a message from mhdproj_last_error(NULL).
 * grid->periodic is honoured: on a periodic axis the high face of the last
 * cell is read at face 0.  All calls on a device share the array: calls that
 * overlap on the GPU race.  The first call on each device looks up the
 * array's device address.  Every call waits on the host for its result, so
 * it cannot be made on a stream that is being captured into a CUDA graph. */
int mhdproj_divergence_noalloc(const mhdproj_grid *grid, const uint8_t *solid, const float *u, const float *v,
                               const float *w, double *out, void *stream);

/* ------------------------------------------------------------ fluid step
 * Fields, diagnostics and the fluid time step around the projection. */

/* FluidDiagnostics (src/fluid/mod.rs:84-96) plus the two reductions the next
 * step's CFL test reads (force_max and max_face_speed, :1140-1141). */
typedef struct {
    float max_speed_m_s;        /* max |cell-centred velocity| */
    float max_divergence_s_inv; /* max |div u| */
    float rms_divergence_s_inv; /* sqrt(sum div^2 / fluid cells) */
    float max_pressure_pa;      /* max |p| */
    float kinetic_energy_j;     /* sum 1/2 rho (face speeds^2) h^3 */
    float fluid_mass_kg;        /* rho_l * sum melt fraction * h^3 */
    float net_flux_m3_s;        /* sum div * h^3 */
    float max_force_density;    /* max |rho_l g + f_em|, N/m^3 */
    float max_face_speed_m_s;   /* max |u| over the faces of fluid cells */
    uint32_t nonfinite_cells;   /* cells with non-finite or out-of-range fields */
    uint32_t viscous_substeps;  /* FluidDiagnostics::viscous_substeps of the last step */
} mhdproj_diagnostics;

/* fields + diagnostics of src/fluid/solver.wgsl:256-291, as dispatched after
 * every accepted step and solid/phase update (src/fluid/mod.rs:899-905,
 * :1311-1317): for the face velocities u, v, w (device arrays) and the
 * context's last pressure potential, the FluidCell record of every cell
 * (cells: 16 floats per cell, velocity xyz + speed, pressure + divergence,
 * force = rho_l a + f_em, reserved (fluid flag, phase fraction, liquid
 * fraction, 0); NULL to skip) and the diagnostics.  em_force: device array of
 * 4 floats per cell holding the EM force density in xyz (NULL: none);
 * acceleration: body acceleration (m/s^2); dt scales the pressure
 * (p = rho_l phi / dt).  Returns MHDPROJ_ERR_NONFINITE with "Nonfinite fluid
 * fields; state restored" when a field is non-finite or out of range (the
 * outputs are still written). */
int mhdproj_fields(mhdproj_ctx *ctx, const float *u, const float *v, const float *w, const float *em_force,
                   const float acceleration[3], float dt, float *cells, mhdproj_diagnostics *diagnostics);

typedef struct {
    float dt;                  /* FluidConfig::dt_s */
    float acceleration[3];     /* FluidConfig::acceleration_m_s2 */
    float kinematic_viscosity; /* nu, m^2/s (Params.physical.z) */
    int32_t advection;         /* FluidConfig::advection: semi-Lagrangian RK2 momentum transport */
    /* moving interface only (two-phase density): */
    float surface_tension;     /* sigma, N/m (Params.surface.z) */
    float air_viscosity;       /* dynamic viscosity of the air, Pa s (Params.surface.w) */
    uint32_t max_viscous_substeps; /* FluidConfig::max_viscous_substeps (0: 4096) */
    const float *curvature;    /* interface curvature per cell, 1/m (reserved.w), device array or NULL */
} mhdproj_step_params;

/* FluidState::step (src/fluid/mod.rs:1246-1333): the velocity CFL test on
 * the previous fields ("Fluid timestep exceeds the velocity CFL limit; reduce
 * Δt"), predict, viscous (body and EM force, mobility), the warm-started
 * projection, fields and diagnostics.  Without a moving interface (one
 * density: reference solver with two_phase = 0, GB300 solver with rho_air =
 * rho_liquid) predict advects (semi-Lagrangian RK2) and viscous adds the
 * explicit viscous term.  With one (reference solver two_phase = 1, GB300
 * solver rho_air != rho_liquid) the momentum is not advected here (the
 * interface transport does it), the capillary / conservative CFL test applies
 * ("Moving-interface capillary or conservative CFL limit exceeded; reduce
 * common timestep"), the Newtonian stresses diffuse the predicted velocity
 * by explicit Euler substeps or damped RKC2 stages
 * (diffuse_surface_stress, :1160-1240; "Viscosity requires N equivalent Euler
 * substeps, above the M work limit; ..."), and viscous adds the capillary
 * force from the curvature with face densities.  u, v, w: device face
 * arrays, the velocity in and the projected velocity out; p_out (cell array)
 * and cells (16 floats per cell, written only when the step is accepted) are
 * optional outputs.  On any error the velocity and p_out are restored to
 * their values on entry, as the reference rolls back its buffers.  The CFL inputs come from the context's last
 * fields pass (mhdproj_fields or the previous step); a context without one
 * first runs a fields pass over the velocity it is given. */
int mhdproj_fluid_step(mhdproj_ctx *ctx, float *u, float *v, float *w, const float *em_force,
                       const mhdproj_step_params *params, float *p_out, float *cells, mhdproj_stats *stats,
                       mhdproj_diagnostics *diagnostics);

/* RunState::export_fields (src/run/export.rs:9-60) for the fluid: writes the
 * cell records (device array of 16 floats per cell, as filled by
 * mhdproj_fields or mhdproj_fluid_step) to <directory>/fluid.bin unchanged
 * (x fastest, then y, then z; host byte order) and publishes
 * <directory>/metadata.json (format_version 1, step, time_s, origin_m,
 * cell_m, dims, byte_order, cell_order, files, moving_interface,
 * forcing_kind) last, by renaming metadata.writing.  The directory must be
 * new ("Create new frame directory <dir>: <reason>" otherwise, read with
 * mhdproj_last_error(NULL)); on any failure the directory created by the call
 * is removed.  origin_m may be NULL (zeros); forcing_kind NULL means "none". */
int mhdproj_export_fields(const mhdproj_grid *grid, const float *cells, const char *directory, uint64_t step,
                          double time_s, const float origin_m[3], int moving_interface, const char *forcing_kind);

/* Fluid mobility and cell phase lanes: the `phase` and `surface` passes of
 * src/fluid/phase.wgsl:10-31 as FluidState::update_cells runs them
 * (src/fluid/mod.rs:713-852).  Device arrays, n = nx*ny*nz cells:
 *   materials   material id per cell; liquid_material = FluidConfig::material_id
 *   thermal     the thermal phase's liquid fraction, read at thermal[i*thermal_stride]
 *               (16 with the reference's thermal packet offset to state.y); NULL: none
 *   interface   NULL runs `phase`; else (a, y) at interface[i*interface_stride + 0/1]
 *               (4 for the reference's vec4 interface field)
 *   mask        0/1 mobility per cell, updated in place
 *   cells       16-float FluidCell records: `phase` writes reserved.y (float 13),
 *               `surface` writes reserved = (1, f, a, y) (floats 12-15)
 *   flags_device one u32 of device scratch
 * *changed: bit 0 some cell's mobility changed (the caller relabels the
 * topology, as update_cells does), bit 1 an interface fraction was outside
 * [-1e-5, 1+1e-5] or not finite, which also returns MHDPROJ_ERR_INVALID with
 * the reference's message (mhdproj_classify_last_error()).  Allocates nothing;
 * synchronises `stream`. */
int mhdproj_classify_cells(const mhdproj_grid *grid, const uint32_t *materials, uint32_t liquid_material,
                           const float *thermal, uint32_t thermal_stride, const float *interface,
                           uint32_t interface_stride, uint32_t *mask, float *cells, uint32_t *flags_device,
                           uint32_t *changed, void *stream);
const char *mhdproj_classify_last_error(void);

/* Host utilities, mirroring src/fluid/multigrid.rs:25-65 and src/fluid/mod.rs:1447-1493. */
/* Aggregation hierarchy: halve (ceil) until every dimension is <= 4.  Returns
 * 0 and the level count / coarse-cell total, or MHDPROJ_ERR_INVALID for zero,
 * overflowing or out-of-range dimensions. */
int mhdproj_hierarchy(const uint32_t dims[4], uint32_t *levels, uint64_t *coarse_cells);
/* Connected components of a 0/1 fluid mask with one root per component;
 * encodes mask[i] = class | root << 2 (class 1 member, 2 root).  Returns the
 * component count. */
uint32_t mhdproj_anchors(uint32_t *mask, const uint32_t dims[3], uint32_t periodic);

/* ---------------------------------------------------------------------------
 * EM induction step: replaces EmState::advance_to (src/em/mod.rs:863-1090)
 * with its passes in src/em/induction.wgsl.
 *
 * The magnetic vector potential lives on the grid's edges: x-edges
 * (nx x (ny+1) x (nz+1)), then y-edges, then z-edges, each block x-fastest
 * (src/em/common.wgsl:3-6).  A step solves the backward-Euler curl-curl
 * system for the reaction potential with Jacobi-preconditioned CG, computes
 * B, J, the Lorentz force J x B and Joule heat per cell, and commits or rolls
 * back.  The applied potential A_s of coils and magnets is an input, which
 * mhdproj_em_evaluate_sources computes from the source elements (the
 * reference's source pass, src/em/source.wgsl); so is the motional EMF
 * (src/em/motion.wgsl, or mhdproj_em_set_motion from the fluid's cell
 * records).  The nodal gradient correction (src/em/nodal.wgsl) takes
 * over after nodal_switch_after Jacobi iterations as in the reference.
 * mhdproj_em_body_forces gives the per-body integrals.
 * ------------------------------------------------------------------------- */
typedef struct mhdproj_em_ctx mhdproj_em_ctx;

typedef enum {
    MHDPROJ_EM_INDUCTION = 0,   /* Mode::Induction: conductors, time steps */
    MHDPROJ_EM_APPLIED = 1      /* Mode::Applied: every cell is vacuum, initial solves only */
} mhdproj_em_mode;

typedef struct {
    uint32_t nx, ny, nz;
    float cell_m;               /* GridSi::cell_m */
    float origin_m[3];          /* GridSi::origin_m (edge positions for applied fields) */
    double dt_s;                /* EmConfig::dt_s */
    float relative_tolerance;   /* EmConfig::relative_tolerance */
    uint32_t max_iterations;    /* EmConfig::max_iterations */
    int32_t mode;               /* mhdproj_em_mode */
    uint32_t nodal_switch_after;/* Jacobi iterations before the nodal gradient correction takes over
                                   (1024 in the reference, src/em/mod.rs:892; 0 = from the first pass) */
} mhdproj_em_config;

/* Diagnostics (src/em/mod.rs:33-46) and the solver's status record. */
typedef struct {
    float maxima[4];            /* max |B| T, |J| A/m^2, |J x B| N/m^3, heat W/m^3 */
    float force_n[3];           /* sum of J x B over the cells, N */
    float power_w;              /* Joule power, W */
    float divergence_j_scaled;  /* max |div J| h^2 per cell, A */
    float max_edge_j;           /* max |J| on an edge */
    float divergence_b_scaled;  /* max |div B| h, T */
    float magnetic_energy_j;
    float applied_max_t;
    float reaction_max_t;
    uint32_t iterations;
    float relative_residual;    /* sqrt(rr / bb) of the accepted solve */
    float conductivity_range[2];/* min sigma > 0 and max sigma over edges, S/m */
    float device_ms;            /* device time of the step */
    double elapsed_ms;          /* host time of the call */
    float status[8];            /* (rz, rr, bb, threshold, alpha, beta, iterations, state) */
} mhdproj_em_diagnostics;

/* Arrays mhdproj_em_copy can read. */
typedef enum {
    MHDPROJ_EM_REACTION = 0,            /* accepted reaction potential, E floats */
    MHDPROJ_EM_PREVIOUS = 1,            /* previous accepted reaction potential, E floats */
    MHDPROJ_EM_APPLIED_POTENTIAL = 2,   /* applied potential A_s, E floats */
    MHDPROJ_EM_CELLS = 3,               /* per cell (B,|B|, J,|J|, JxB,heat, applied B,|applied B|), 16 floats */
    MHDPROJ_EM_WORK = 4,                /* per edge (x, r, p, w) as the reference's work record, 4 floats */
    MHDPROJ_EM_EDGE_COEFFICIENTS = 5    /* per edge (sigma, diagonal, flags, motional EMF), 4 floats */
} mhdproj_em_array;

int mhdproj_em_create(const mhdproj_em_config *config, mhdproj_em_ctx **out);
/* Takes dt_s, relative_tolerance, max_iterations and nodal_switch_after from
 * `config` for the following steps (the EmConfig fields the reference lets a
 * caller change); the grid, origin and mode stay as created. */
int mhdproj_em_update_config(mhdproj_em_ctx *ctx, const mhdproj_em_config *config);
void mhdproj_em_destroy(mhdproj_em_ctx *ctx);
const char *mhdproj_em_last_error(const mhdproj_em_ctx *ctx);
int mhdproj_em_set_stream(mhdproj_em_ctx *ctx, void *stream);
/* out: nx, ny, nz, cells, x-edges, y-edges, z-edges, edges. */
int mhdproj_em_sizes(const mhdproj_em_ctx *ctx, uint64_t out[8]);
/* Material ids per cell (device; bit 31 marks a partial cell whose fraction
 * is in bits 8..30 and material in bits 0..7) with (conductivity S/m,
 * relative permeability) rows per id (host, `count` rows, row 0 = the
 * background).  Builds the edge coefficients (coefficients +
 * coefficient_check, induction.wgsl:105-131; also clears the motional EMF).
 * Fails with the reference's message when a conductor touches the outer
 * boundary (mod.rs:563-567). */
int mhdproj_em_set_materials(mhdproj_em_ctx *ctx, const uint32_t *materials, const float *properties,
                             uint32_t count, float conductivity_range[2]);
/* Motional EMF per edge (device, E floats; NULL clears it). */
int mhdproj_em_set_motional_emf(mhdproj_em_ctx *ctx, const float *emf);
/* The energy ledger of the last committed step (EmState::energy_step,
 * src/em/mod.rs:1106-1133, energy.wgsl), joules: out = (magnetic, change of
 * magnetic, backward-Euler loss, Joule heat, mechanical work, external work,
 * balance error = external - the other four).  At time 0 only the magnetic
 * energy is reported. */
int mhdproj_em_energy(mhdproj_em_ctx *ctx, double out[7]);
/* Per-body force (N, xyz) and Joule power (W) of the last accepted step
 * (body-stats.wgsl, src/em/mod.rs:1036-1069): body z holds the cells with
 * bit z of masks[i] set (device, one u32 per cell; 1 <= bodies <= 32).
 * totals: 4 floats per body, host memory. */
int mhdproj_em_body_forces(mhdproj_em_ctx *ctx, const uint32_t *masks, uint32_t bodies, float *totals);
/* The source pass (src/em/source.wgsl): the applied potential A_s at every
 * edge midpoint of `count` source elements as EmConfig::elements builds them
 * (src/em/sources.rs:280-338), 12 floats each (a, b, c as vec4; host
 * memory).  c.y selects the kind: < 0.5 a wire segment from a to b with core
 * radius c.x carrying c.z amperes; < 1.5 a surface-current element at a with
 * moment b scaled by c.z, softening c.x; otherwise a uniform field b tesla
 * scaled by c.z.  Elements with c.z == 0 contribute nothing.  Summed in
 * batches of 32 elements as the reference's passes are.  Writes E floats to
 * `applied` (device), ready for mhdproj_em_advance.  Fails with the
 * reference's messages for more than 1e6 elements, non-finite values, or
 * more than 5e10 edge-element pairs. */
int mhdproj_em_evaluate_sources(mhdproj_em_ctx *ctx, const float *elements, uint32_t count, float *applied);
/* The motional EMF of EmState::set_velocity (src/em/mod.rs:757-834,
 * motion.wgsl): per edge the conductivity-weighted u x B of the four cells
 * around it, from the fluid's 16-float cell records (velocity floats 0-2,
 * mobile where float 12 > 0.5; device, cells x 16) and the B of the last
 * accepted EM step, with the conductivities of the last material update. */
int mhdproj_em_set_motion(mhdproj_em_ctx *ctx, const float *fluid_cells);
/* Overwrites the accepted reaction potential (device, E floats). */
int mhdproj_em_set_reaction(mhdproj_em_ctx *ctx, const float *a);
/* One step to time_s (initial != 0: the source-only solve EmState::new and
 * evaluate_applied run).  applied: A_s at time_s (device, E floats), or NULL
 * when the applied field is unchanged.  On failure the state is restored. */
int mhdproj_em_advance(mhdproj_em_ctx *ctx, double time_s, int initial, const float *applied,
                       mhdproj_em_diagnostics *diagnostics);
/* Copies one mhdproj_em_array into `out` (device). */
int mhdproj_em_copy(mhdproj_em_ctx *ctx, int which, float *out);
/* q = A p with (air_stencil != 0) or without the seven-point air stencil
 * (the operator check of src/em/tests.rs:666-738). */
int mhdproj_em_apply_operator(mhdproj_em_ctx *ctx, const float *p, float *q, int air_stencil);
int mhdproj_em_kernel_launches(const mhdproj_em_ctx *ctx, uint64_t *count);

#ifdef __cplusplus
}
#endif
#endif
