/*
 * mhd_oracle.h -- CPU oracle for the MAC pressure projection.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links this code;
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it,
 * and only as the expected results the GPU path is compared with or as the
 * timed CPU baseline.
 *
 * Two parts:
 *
 *  oref_*  A line-by-line FP32 restatement of the reference projection as it
 *          runs in the reference's WGSL shaders (src/fluid/solver.wgsl,
 *          src/fluid/multigrid.wgsl, src/fluid/pressure_subspace.wgsl,
 *          src/periodic.wgsl) driven by the host logic of
 *          src/fluid/mod.rs:969-1115 and src/fluid/multigrid.rs:25-329.
 *          Buffers keep the reference layout (vec4 per (n+1)^3 face-cell,
 *          vec4 work per cell).  Workgroup reductions are replayed in the
 *          reference's order (256-lane tree, then a 256-stride final pass).
 *
 *  onat_*  An FP64 solver for the GB300 path's own discrete problem
 *          (two-phase mobility, solid walls, optional Dirichlet outlet on the
 *          top z-face, pinned gauges for components without an outlet) and
 *          its adjoint.  The face mobilities are computed in FP32 with the
 *          same operation order as the GPU, then the system is solved in FP64
 *          to a 1e-13 relative residual.
 *
 * Parity status: the reference runs only through wgpu/Vulkan, which neither
 * this machine nor the GPU machine can run, so the restatement is pinned by the
 * reference's own known-answer tests (hierarchy sizes, gauge anchors) and its
 * analytic acceptance tests (periodic cosine potential, manufactured gradient,
 * Galerkin identity, V-cycle symmetry, fused coarse solve, cached/uncached
 * operator) -- not by stored reference output vectors, which do not exist.
 */
#ifndef MHD_ORACLE_H
#define MHD_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- reference */

/* Projection lanes of Params (src/fluid/mod.rs:120-130). */
typedef struct {
    uint32_t dims[4];    /* nx, ny, nz, n */
    uint32_t faces[4];   /* nx+1, ny+1, nz+1, nf */
    uint32_t flags[4];   /* x periodic bits, w thermal-phase drag enabled */
    float physical[4];   /* h, dt, nu, rho_liquid */
    float initial[4];    /* w: inverse fluid-cell count in mean-free mode */
    float solve[4];      /* tol^2, absolute floor, bound, mushy drag rate */
    float surface[4];    /* x enabled, y rho_air */
} oref_params;

typedef struct {
    int32_t status;        /* 0 ok, 1 not converged, 2 non-finite, 3 no progress */
    uint32_t iterations;
    float residual;        /* sqrt(s[1]/s[2]) of the last convergence read */
    int32_t meanfree;      /* gauge mode chosen by configure_pressure_projection */
    int32_t multigrid;     /* preconditioner used */
    uint32_t levels;       /* multigrid levels (0 when Jacobi) */
    uint64_t coarse_cells;
} oref_result;

/* anchors(): src/fluid/mod.rs:1447-1493.  mask in: 0/1; out: encoded. */
uint32_t oref_anchors(uint32_t *mask, const uint32_t dims[3], uint32_t periodic_bits);

/* hierarchy(): src/fluid/multigrid.rs:25-65.  Returns 0 on success and fills
 * the number of levels and total coarse cells; nonzero for rejected dims. */
int oref_hierarchy(const uint32_t dims[4], uint32_t *levels, uint64_t *coarse_cells,
                   uint32_t *level_dims /* 4*levels, may be NULL */, uint32_t max_levels);

/* Fill Params the way FluidState::new + configure_pressure_projection do. */
void oref_make_params(oref_params *p, const uint32_t dims[3], float h, float dt,
                      float rho_liquid, float rho_air, int two_phase, uint32_t periodic_bits,
                      float rel_tol, float abs_div_tol, uint32_t fluid_cells,
                      int thermal_drag, float drag_rate);

/* FluidState::project(warm_start) (src/fluid/mod.rs:1015-1115) with the
 * configure/gauge selection of :978-1002.
 *   force_mg: -1 automatic (cells >= 96^3), 0 Jacobi-CG, 1 aggregation MG-CG
 *   force_meanfree: -1 automatic (components == 1), 0 pinned, 1 mean-free if connected
 *   predicted: vec4[nf] candidate face velocities (modified by a warm start)
 *   velocity:  vec4[nf] out: projected face velocities
 *   work:      vec4[n]  out: x = pressure potential
 *   occupancy: liquid fraction per cell (FluidCell.reserved.z)
 *   phase:     phase fraction per cell (FluidCell.reserved.y) or NULL
 *   old_pressure: FluidCell.pressure.x per cell for warm_start, else NULL */
void oref_project(const oref_params *params, const uint32_t *mask, uint32_t components,
                  const float *occupancy, const float *phase, const float *old_pressure,
                  float *predicted, float *velocity, float *work, uint32_t max_iterations,
                  int warm_start, int force_mg, int force_meanfree, oref_result *result);

/* Fluid step without a moving interface (FluidState::step,
 * src/fluid/mod.rs:1246-1333): predict (solver.wgsl:127-141; flags[1] =
 * semi-Lagrangian RK2 advection), viscous (:143-163 with surface.x = 0;
 * physical[2] = kinematic viscosity), then fields and diagnostics
 * (:256-291).  Face buffers are vec4[nf]; em is vec4 per cell (force density
 * in .xyz) or NULL; reserved_in vec4 per cell or NULL; cells 16 floats per
 * cell or NULL; scalars the 12 diagnostics floats (max speed, max |div|,
 * sum div^2, kinetic energy, max |p|, sum div, max |force|, bad cells, max
 * face speed, melt sum, 0, 0). */
void oref_predict(const oref_params *params, const uint32_t *mask, const float *velocity, float *predicted);
void oref_viscous(const oref_params *params, const uint32_t *mask, const float *occupancy, const float *phase,
                  const float *em, const float acceleration[3], const float *predicted, float *velocity);
/* viscous() with a moving interface (surface.x = 1): face density, capillary
 * force sigma k (alpha_R - alpha_L) / h from the per-cell curvature (or
 * NULL), mobility times rho_face / rho_l, no explicit Laplacian. */
void oref_viscous_surface(const oref_params *params, const uint32_t *mask, const float *occupancy, const float *phase,
                          const float *em, const float acceleration[3], const float *curvature, float sigma,
                          const float *predicted, float *velocity);
/* FluidState::diffuse_surface_stress (src/fluid/mod.rs:1160-1240): Euler
 * substeps or damped RKC2 stages of the Newtonian stress operator of
 * src/fluid/viscosity.wgsl on `predicted` (in/out); `velocity` holds the
 * step's starting velocity and serves as the second stage buffer.  Returns 0,
 * 1 (non-finite bound) or 2 (more substeps than max_substeps). */
int oref_diffuse_surface_stress(const oref_params *params, const uint32_t *mask, const float *occupancy,
                                const float *phase, float mu_air, float dt, uint32_t max_substeps,
                                float *predicted, float *velocity, uint32_t *substeps, float *gpu_bound);
/* stabilized::schedule: rows of 8 floats; returns the row count. */
uint32_t oref_rkc_schedule(double dt, uint32_t euler_steps, float *rows, uint32_t cap);
void oref_fields(const oref_params *params, const uint32_t *mask, const float *occupancy, const float *work,
                 const float *velocity, const float *em, const float acceleration[3], const float *reserved_in,
                 float *cells, float scalars[12]);

/* pressure_coefficients (solver.wgsl:93-103) into velocity vec4[nf]. */
void oref_coefficients(const oref_params *params, const uint32_t *mask, const float *occupancy,
                       const float *phase, float *velocity);
/* apply() (cached, solver.wgsl:78-92) and laplacian()/diagonal() (uncached,
 * :60-69) for every fluid cell; kind 0 reads work.x, 1 reads work.z. */
void oref_apply_cached(const oref_params *params, const uint32_t *mask, const float *velocity,
                       const float *work, uint32_t kind, float *out);
void oref_apply_uncached(const oref_params *params, const uint32_t *mask, const float *occupancy,
                         const float *phase, const float *work, uint32_t kind, float *out,
                         float *diag_out);

/* Aggregation multigrid probes (multigrid.wgsl) on a prepared fine state:
 * velocity holds the coefficient cache, work the fine vectors. */
typedef struct oref_mg oref_mg;
oref_mg *oref_mg_create(const oref_params *params, const uint32_t *mask, const float *velocity,
                        int meanfree);
void oref_mg_destroy(oref_mg *mg);
uint32_t oref_mg_levels(const oref_mg *mg, uint32_t *level_dims /* 4 per level */,
                        uint32_t *offsets /* per level */);
void oref_mg_build(oref_mg *mg);
/* The fixed V-cycle: work.y (residual) -> work.w (correction). */
void oref_mg_apply(oref_mg *mg, float *work);
/* Direct access for probes: coarse coeff/value vec4 buffers. */
float *oref_mg_coeff(oref_mg *mg);
float *oref_mg_value(oref_mg *mg);
/* probe_action (multigrid_probes.wgsl:7) at a level; fine results go to
 * predicted_w[n], coarse results to value.z. */
void oref_mg_probe_action(oref_mg *mg, uint32_t level, const float *work, float *predicted_w);
/* coarse_solve at the coarsest level vs. the clear + 8 smooth ping-pongs. */
void oref_mg_coarse_solve(oref_mg *mg, float *work);
void oref_mg_coarse_jacobi_sequence(oref_mg *mg, float *work);

/* ------------------------------------------------------------------- native */

typedef struct {
    uint32_t nx, ny, nz;
    uint32_t periodic;     /* bit a: axis a periodic */
    int32_t outlet;        /* 1: Dirichlet p=0 on the top z-face */
    float h;
    float rho_liquid, rho_air;
    int32_t single;        /* one phase: face mobility 1 (SurfaceConfig disabled) */
    float drag_rate, dt;   /* thermal phase drag (with phase) */
    const float *phase;    /* thermal phase fraction per cell, or NULL: no drag */
} onat_grid;

/* Cell classes: 0 solid, 1 active fluid, 2 pinned gauge cell.  Components that
 * touch an outlet face get no gauge; every other component is pinned at its
 * first cell in x-fastest order (the root the reference's anchors() picks). */
uint32_t onat_classify(const onat_grid *g, const uint8_t *solid, uint8_t *cls);

/* Low-face mobilities and reactions, FP32, coef[4*n] = (bx, by, bz, reaction);
 * gtop[nx*ny] = outlet conductance 2*rho_l/rho(cell) (0 without an outlet). */
void onat_coefficients(const onat_grid *g, const float *alpha, const uint8_t *cls, float *coef,
                       float *gtop);
/* b = -h * sum of open-face velocity differences (FP64). */
void onat_rhs(const onat_grid *g, const uint8_t *cls, const float *gtop, const float *u,
              const float *v, const float *w, double *b);
void onat_apply(const onat_grid *g, const float *coef, const double *x, double *y);
/* FP64 PCG (symmetric Gauss-Seidel preconditioner) to ||b-Ax|| <= rtol ||b||. */
int onat_solve(const onat_grid *g, const float *coef, const uint8_t *cls, const double *b,
               double *x, double rtol, int max_it, int *iterations, double *rel_residual);
/* Gradient subtraction: out = u* - beta * grad(phi) / h, 0 on closed faces. */
void onat_correct(const onat_grid *g, const float *alpha, const uint8_t *cls, const float *gtop,
                  const double *phi, const float *us, const float *vs, const float *ws,
                  double *u, double *v, double *w);
/* Whole projection in FP64; pressure p = rho_l * phi / dt. */
int onat_project(const onat_grid *g, const float *alpha, const uint8_t *solid, const float *us,
                 const float *vs, const float *ws, float dt, double rtol, double *phi, double *u,
                 double *v, double *w, double *p, int *iterations, double *rel_residual);
/* Vector-Jacobian product of the projection: given dL/du (faces) and dL/dp
 * (cells, may be NULL) return dL/du* (faces). */
int onat_project_vjp(const onat_grid *g, const float *alpha, const uint8_t *solid, const double *gu,
                     const double *gv, const double *gw, const double *gp, float dt, double rtol,
                     double *gus, double *gvs, double *gws);
/* Coarse-correction weight of the V-cycle used as the FP64 preconditioner. */
void onat_set_prolongation(double w);
/* Max and RMS cell divergence sum(u_high-u_low)/h over active cells. */
void onat_divergence(const onat_grid *g, const uint8_t *cls, const float *gtop, const double *u,
                     const double *v, const double *w, double *max_abs, double *rms);

/* Chain u_{k+1} = P(u_k + dt f / rho_face), J = sum over outlet faces of w^2.
 * Forward returns J; the adjoint returns dJ/df on the faces. */
int onat_chain_forward(const onat_grid *g, const float *alpha, const uint8_t *solid,
                       const float *u0, const float *v0, const float *w0, const float *fu,
                       const float *fv, const float *fw, float dt, int steps, double rtol,
                       double *uk, double *vk, double *wk, double *objective);
int onat_chain_adjoint(const onat_grid *g, const float *alpha, const uint8_t *solid,
                       const double *uk, const double *vk, const double *wk, float dt, int steps,
                       double rtol, double *gfu, double *gfv, double *gfw);
/* The same chain with J = sum over the states u_1 .. u_K of the outlet term
 * (all states kept in FP64); dJ/df into gf* when they are not NULL. */
int onat_chain_summed(const onat_grid *g, const float *alpha, const uint8_t *solid, const float *u0,
                      const float *v0, const float *w0, const float *fu, const float *fv, const float *fw, float dt,
                      int steps, double rtol, double *objective, double *gfu, double *gfv, double *gfw);

/* phase / surface passes (src/fluid/phase.wgsl:10-31): mobility mask and
 * FluidCell.reserved lanes; returns the changed flags (bit 0 mobility, bit 1
 * an interface fraction out of range). interface == NULL: the phase pass. */
uint32_t oref_classify_cells(uint32_t n, const uint32_t *materials, uint32_t liquid, const float *thermal,
                             uint32_t thermal_stride, const float *interface, uint32_t interface_stride,
                             uint32_t *mask, float *cells);

/* ---- oem_*: the implicit EM induction solve (oracle_em.c) ----
 * FP32 restatement of the reference's edge-element A-formulation step:
 * src/em/induction.wgsl (coefficients, Jacobi-preconditioned CG with
 * power-of-two residual scaling, true-residual restarts, fields) driven by
 * EmState::advance_to (src/em/mod.rs:863-1090).  Edges are numbered x-edges,
 * y-edges, z-edges, each block x-fastest (src/em/common.wgsl:3-6). */
typedef struct OEm OEm;
enum { OEM_OK = 0, OEM_NOT_CONVERGED = 1, OEM_NONFINITE = 2 };
/* vacuum != 0 is the applied-field mode (every cell reads as air). */
OEm *oem_new(const uint32_t dims[3], float h, const float origin[3], double dt_s, float rel_tol, uint32_t max_it,
             int vacuum);
void oem_free(OEm *s);
/* out: dims[4] (nx, ny, nz, cells), edges[4] (x, y, z, total). */
void oem_sizes(const OEm *s, uint32_t out[8]);
/* Material ids per cell (bit 31: partial cell, fraction in bits 8..30,
 * material in bits 0..7) and (sigma S/m, relative permeability) per id.
 * check = (conducting boundary edges, min sigma>0, max sigma, conducting
 * edges).  Returns -1 when an id has no property row. */
int oem_set_materials(OEm *s, const uint32_t *materials, const float *props, uint32_t n_props, float check[4]);
/* Motional EMF per edge (NULL: zero), as set_velocity leaves it. */
void oem_set_motional(OEm *s, const float *emf);
/* Iterations before the solve switches to the nodal correction (1024 in the
 * reference; 0 = from the first pass, the reference's test setting). */
void oem_set_nodal_switch(OEm *s, uint32_t after);
/* The mutable EmConfig fields (dt_s, relative_tolerance, max_iterations). */
void oem_update_config(OEm *s, double dt_s, float rel_tol, uint32_t max_it);
/* The reference's test switch predict_increments, its prediction_diagnostic
 * (factor, initial relative residual, fallback flag) and (time, last dt). */
void oem_set_predict(OEm *s, int on);
/* The nodal-corrected preconditioner applied to a residual (edges). */
void oem_apply_nodal(OEm *s, const float *r, float *out);
/* Overwrite the previous accepted potential (the tests' poisoned history). */
void oem_set_previous(OEm *s, const float *a);
void oem_prediction(const OEm *s, float out[3]);
void oem_time(const OEm *s, double out[2]);
/* Applied potential of source elements (12 floats each) at the edges
 * (the source pass, source.wgsl); out: E floats. */
void oem_evaluate_sources(const OEm *s, const float *elements, uint32_t count, float *out);
/* Energy ledger of the last committed step (energy.wgsl): magnetic, delta
 * magnetic, backward-Euler loss, Joule, mechanical, external, balance (J).
 * Returns -1 for a non-finite integral. */
int oem_energy(OEm *s, double out[7]);
/* Per-body force (N) and Joule power (W) from the last cell results; body z
 * holds the cells with bit z of masks[i] (body-stats.wgsl). totals: 4/body. */
void oem_body_forces(const OEm *s, const uint32_t *masks, uint32_t bodies, float *totals);
/* Motional EMF from fluid cell records (set_velocity, motion.wgsl). */
void oem_set_motion(OEm *s, const float *fluid_cells);
/* Overwrite the accepted reaction potential (edges). */
void oem_set_reaction(OEm *s, const float *a);
/* which: 0 work (E x 4), 1 previous (E), 2 source (2E x 4), 3 cell results
 * (cells x 16: B,|B|, J,|J|, F,heat, applied B,|applied B|), 4 scalars (32). */
void oem_get(const OEm *s, int which, float *out);
/* q = A p with (use_air = 1) or without the air stencil fast path. */
void oem_apply_operator(OEm *s, const float *p, float *q, int use_air);
/* One step to time_s; applied = A_s at that time (NULL: unchanged).
 * Returns OEM_*; status_out = scalars[0..1], stats_out = scalars[2..5]. */
int oem_advance(OEm *s, double time_s, int initial, const float *applied, float status_out[8], float stats_out[16]);

#ifdef __cplusplus
}
#endif
#endif
