// kernels.h -- host-side launchers of the projection kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "common.cuh"

namespace mhdproj {

struct Launch {
    dim3 grid, block;
    Grid3 g;
    int nblocks;
};
// 32x8 tiles over (x, y), z split into runs so that about `target` blocks run.
Launch tile_launch(int nx, int ny, int nz, int periodic, int target_blocks);

struct Fields {
    // GB300 solver fine-level state (all device pointers)
    const uint8_t* cls;
    const float* alpha;
    float4* coef;
    void* coef_lo;     // FP16/BF16 copy (mixed precision) or nullptr
    int coef_lo_kind;  // 0 none, 1 fp16, 2 bf16
    float* gtop;
    float *b_hi, *b_lo;
    float *r, *z, *p, *q, *e;
    Scalars* sc;
    double* partials;
    int outlet;
    float h, rho_l, rho_air;
    Mobility mob;  // face mobility (densities, one-phase flag, thermal drag)
    long long n_active;
};

// ---- GB300 solver kernels (gb300_kernels.cu)
void launch_coefficients(const Launch& L, const Fields& F, cudaStream_t s);
void launch_init_scalars(Scalars* sc, double tol2, double abs_floor, double inner_floor2, int max_total,
                         cudaStream_t s);
// start_pass: also r = b, x = 0 and the first pass's scalars (a solve from x = 0)
void launch_rhs(const Launch& L, const Fields& F, const float* u, const float* v, const float* w, cudaStream_t s,
                bool start_pass = false);
void launch_residual(const Launch& L, const Fields& F, const float* x_hi, const float* x_lo, cudaStream_t s);
void launch_spmv_pq(const Launch& L, const Fields& F, cudaStream_t s);
void launch_update(const Launch& L, const Fields& F, cudaStream_t s);
void launch_dot_rz(const Launch& L, const Fields& F, int init, cudaStream_t s);
void launch_search(const Launch& L, const Fields& F, cudaStream_t s);
void launch_accumulate(const Launch& L, const Fields& F, float* x_hi, float* x_lo, cudaStream_t s);
void launch_to_double(const float* hi, const float* lo, double* out, long long n, cudaStream_t s);
void launch_correct(const Launch& L, const Fields& F, const float* ph, const float* pl, const float* us,
                    const float* vs, const float* ws, float* uo, float* vo, float* wo, float* po, float dt,
                    cudaStream_t s);
void launch_divergence(const Launch& L, const Fields& F, const float* u, const float* v, const float* w,
                       cudaStream_t s);
void launch_apply(const Launch& L, const Fields& F, const float* x, float* y, cudaStream_t s);
void launch_set_sigma(Scalars* sc, float sigma, cudaStream_t s);
// no_stop: also disable the stop test, so repeated launches keep running
void launch_profile_reset(Scalars* sc, cudaStream_t s, bool no_stop = false);
void launch_scale(const Launch& L, const float* in, float* out, float scale, const Scalars* sc, cudaStream_t s);
// adjoint and chain
void launch_adj_rhs(const Launch& L, const Fields& F, const float* gu, const float* gv, const float* gw,
                    const float* gp, float dt, cudaStream_t s);
void launch_adj_correct(const Launch& L, const Fields& F, const float* psi_hi, const float* psi_lo, const float* gu,
                        const float* gv, const float* gw, float* ou, float* ov, float* ow, cudaStream_t s);
void launch_add_force(const Launch& L, const Fields& F, const float* u, const float* v, const float* w,
                      const float* fu, const float* fv, const float* fw, float dt, float* su, float* sv, float* sw,
                      cudaStream_t s);
void launch_force_grad(const Launch& L, const Fields& F, const float* lu, const float* lv, const float* lw, float dt,
                       double* gu, double* gv, double* gw, cudaStream_t s);
// J = sum of w^2 over the outlet faces into the scalars (added to them when
// `accumulate`); seed_w = 2 w on those faces (added when `add_seed`).
void launch_outlet_objective(const Launch& L, const Fields& F, const float* w, float* seed_w, cudaStream_t s,
                             bool accumulate = false, bool add_seed = false);

// ---- finest-level kernels with shared-memory plane staging (fine_kernels.cu)
void launch_spmv_staged(const Launch& L, const Fields& F, cudaStream_t s);
void launch_smooth_staged(int ck, const Launch& L, const void* coef, const float* r, float* e, float* tmp, int color,
                          bool zero, bool out_of_place, const Scalars* sc, cudaStream_t s);
void launch_restrict_staged(int ck, const Launch& L, const Grid3& gc, const void* coef, const float* r, const float* e,
                            void* rc, const Scalars* sc, cudaStream_t s);
cudaError_t staged_prepare_attributes();
bool staged_supported(const Grid3& g);

// ---- multigrid (mg_kernels.cu)
struct MGLevel {
    Launch L;
    float4* coef32;  // FP32 master coefficients (level 0: the fine cache)
    void* coef_lo;   // level-precision copy (nullptr in FP32 mode)
    void* r;         // level residual (level 0: the CG residual, FP32)
    void* e;         // level correction (level 0: the preconditioned residual z, FP32)
    void* tmp;       // half-step scratch for levels with odd periodic extents
    void* eo;        // post-smoothing output of a fused level >= 1 (level precision)
    void* sm;        // smoother records (beta_x, beta_y, beta_z, diagonal) of a fused level
    void* r2;        // second-visit right-hand side of a fused W-cycle level (level precision)
    void* eo2;       // second-visit output of a fused W-cycle level (level precision)
    bool odd_periodic;
};
// The levels of the bottom sub-cycle kernel (shared-memory offsets in floats
// / float4s).
struct BottomLevel {
    Grid3 g;
    int n;
    int off;          // r at off, e at off + n, scratch at off + 2n (floats)
    int coff;         // coefficient records at coff (float4s)
    int xoff;         // packed cell coordinates, red cells first, at xoff (ints, in float units)
    int nred;         // cells of colour 0
    const void* coef; // level-precision records (beta_x, beta_y, beta_z, reaction)
    void* r;          // level residual in global memory (level precision)
    void* e;          // level correction in global memory (level precision)
    bool odd;         // odd periodic extent: half-steps out of place
};
enum { BOP_PRE = 0, BOP_POST, BOP_COARSE, BOP_SAVE_RESID, BOP_ADD_SAVED };
constexpr int BOTTOM_MAX_OPS = 256;
struct BottomPlan {
    int nl;
    BottomLevel lv[8];
    const float* ainv;
    const float4* img;  // shared-memory image (records, cell lists, inverse), built per coefficient set
    int img_floats;     // its size in floats (a multiple of 4)
    int aoff;           // coarsest inverse at aoff (floats)
    int m;
    float w;
    int nops;
    unsigned char ops[BOTTOM_MAX_OPS];  // (op << 4) | level
};
constexpr size_t BOTTOM_SMEM_MAX = 200 * 1024;

struct MGPlan {
    int precision;  // 0 fp32, 1 fp16, 2 bf16
    int nlevels;
    MGLevel lv[32];
    float* ainv;    // dense inverse of the coarsest operator (m x m)
    int m;
    float prolong;  // coarse-correction weight
    Scalars* sc;
    bool staged;    // finest level through the shared-memory staged kernels
    int fused_levels;  // levels 0 .. fused_levels-1 run as fused pre-/post-smoothing passes (0: none)
    int bottom_from;   // levels from here down run in one bottom sub-cycle kernel (0: none)
    int w_from, w_to;  // levels w_from..w_to (>= 1) take two coarse visits, a W-cycle step (0: none)
    bool w_disabled;   // the W-cycle step made the preconditioner indefinite here: V-cycles only
    size_t bottom_smem;
    BottomPlan bottom;
    float4* bottom_img;  // the bottom sub-cycle's shared-memory image (bottom.img_floats floats)
    float* e0;         // fine-level pre-smoothed correction of the fused passes
    int pin_coarse;    // mean-free gauge: the coarsest cell held at zero in the coarsest solve (-1: none)
};
void mg_build(const MGPlan& P, cudaStream_t s);
// single fine-level stages, for measurement
void mg_fine_smooth(const MGPlan& P, int color, cudaStream_t s);
void mg_fine_restrict(const MGPlan& P, cudaStream_t s);
void mg_fine_prolong(const MGPlan& P, cudaStream_t s);
void mg_vcycle(const MGPlan& P, cudaStream_t s);
void mg_vcycle_from(const MGPlan& P, int l0, cudaStream_t s);
void mg_plan_bottom(MGPlan& P);

// ---- pipelined CG with fused V-cycle passes (fused_kernels.cu, fine_kernels.cu)
bool fused_supported(const Grid3& g);
cudaError_t fused_prepare_attributes();
// One V-cycle z = B(sigma r) / sigma through the fused passes; update: the
// residual is first updated, r_out = r_in - alpha q.  Ends with rz and beta.
void mg_vcycle_fused(const MGPlan& P, const float* r_in, const float* q, float* r_out, bool update, double* partials,
                     long long n_active, cudaStream_t s);
void mg_fused_pre(const MGPlan& P, const float* r_in, const float* q, float* r_out, double* partials, cudaStream_t s);
void mg_fused_post(const MGPlan& P, const float* r, double* partials, long long n_active, cudaStream_t s);
void mg_fused_coarse(const MGPlan& P, double* partials, long long n_active, cudaStream_t s);
void mg_bottom_cycle(const MGPlan& P, cudaStream_t s);
// Smoother records of the fused levels, after every coefficient change.
void mg_smoother_records(const MGPlan& P, cudaStream_t s);
void launch_search_spmv(const Launch& L, const float4* coef, const float* z, const float* p_old, float* p_new,
                        float* x, float* q, Scalars* sc, double* partials, int pidx_new, cudaStream_t s);
void launch_accumulate_pipelined(const Launch& L, float* x_hi, float* x_lo, const float* x, const float* p0,
                                 const float* p1, const Scalars* sc, cudaStream_t s);
cudaError_t mg_prepare_attributes();
// The same two passes with TMA-staged planes (tma_fused.cu), for grids without
// periodic axes whose rows are whole 16-byte multiples; they return false, and
// launch nothing, where they do not apply (the cp.async passes then run).
// fine: level 0 (FP32 vectors, the level-precision coarse residual);
// otherwise a coarse level in the level precision.
cudaError_t tma_prepare_attributes();
bool tma_fused_enabled();
bool tma_pre(int ck, bool fine, bool update, const Grid3& g, const Grid3& gc, const void* sm, const void* rin,
             const float* q, float* r_out, void* e, void* rc, Scalars* sc, double* partials, cudaStream_t s);
bool tma_post(int ck, bool fine, const Grid3& g, const Grid3& gc, const void* sm, const void* e, const void* ec,
              const void* r, void* out, const void* accum, float w, Scalars* sc, double* partials, long long n_active,
              cudaStream_t s);

// ---- connected components of the non-solid cells (topology_kernels.cu)
struct TopoCounts {
    unsigned long long components;  // roots (one per component)
    unsigned long long fluid;       // non-solid cells
    unsigned long long pinned;      // gauge cells (classes only)
    int error;                      // a label walk or link hit its bound
    int pad;
};
// labels: u32[n] scratch; roots: u32[(n + 1) / 2] scratch (the most
// components a 6-connected grid can have).  mask_out (optional): the
// reference's encoding (0 solid, 1 | root << 2, 2 | root << 2).  cls_out
// (optional): 0 solid, 1 active, 2 pinned gauge cell, where components that
// reach the top z-layer need no gauge when `outlet` is set on a non-periodic
// z axis; topflag: u8[n] scratch for that case.  counts: components, fluid
// cells and (classes) pinned cells; active = fluid - pinned.  Requires
// n < 2^31.  Returns the kernels launched.
int launch_topology(const uint8_t* solid, int nx, int ny, int nz, int periodic, int outlet, uint32_t* labels,
                    uint32_t* roots, uint8_t* topflag, uint32_t* mask_out, uint8_t* cls_out, TopoCounts* counts,
                    cudaStream_t s);
// ---- fluid step and fields (step_kernels.cu)
struct StepView {
    uint32_t dims[4];       // nx, ny, nz, n
    uint32_t periodic;      // bit a: axis a periodic
    int advection;          // predict: semi-Lagrangian RK2
    int two_phase;          // density from the liquid fraction (fields only in a step)
    int mean_free;          // pressure relative to the component root (reference mask)
    float h, dt, nu, rho_l, rho_air, drag_rate;
    float acc[3];
    const uint32_t* mask;   // reference encoding (fluid != 0), or null
    const uint8_t* cls;     // GB300 classes (fluid != 0) when mask is null
    const float* occ;       // liquid fraction or null
    const float* phase;     // thermal phase fraction (phase drag) or null
    const float* vel[3];    // face arrays read by face()
    const uint8_t* open[3]; // open_face() flags per face position (viscous)
    const float4* em;       // EM force density per cell (xyz) or null
    const float* phi;       // pressure potential, element i at phi[i * phi_stride]
    int phi_stride;
    // moving interface (two_phase): surface tension, air dynamic viscosity,
    // interface curvature per cell (or null), and the stress workspace
    float sigma, mu_air;
    const float* curv;
    float* mu_c;            // cell viscosity cached for a diffusion macro-step
    float4* t4;             // normal stresses xx, yy, zz and shear xy per cell
    float2* t2;             // shear xz, yz per cell
    float4* y0;             // RKC initial face values per cell (lanes x, y, z)
    float4* f0;             // RKC initial stress acceleration per cell
};
// masked / open: three face arrays of scratch each (face() and open_face()
// of every position); viscous reads the open flags through StepView::open
void launch_predict(const StepView& s, float* const out[3], float* const masked[3], uint8_t* const open[3],
                    cudaStream_t st);
void launch_viscous(const StepView& s, float* const out[3], cudaStream_t st);
// Moving-interface stress diffusion (s.vel: the face arrays the stresses
// read).  Cell viscosities into s.mu_c; the shared stress tensor into s.t4/t2;
// RKC initial state into s.y0/f0; one RKC stage out = blend of the stage
// arrays; one explicit Euler substep out = u + dt_sub a(u); the stability
// bound (max over faces) into *bound_bits (float bits, cleared by the caller).
void launch_stress_coefficients(const StepView& s, cudaStream_t st);
void launch_stress_tensor(const StepView& s, cudaStream_t st);
void launch_stress_save_initial(const StepView& s, cudaStream_t st);
// row: mu, nu, 1 - mu - nu, op, initial-operator weight
void launch_stress_stage(const StepView& s, const float row[5], float* const io[3], cudaStream_t st);
// t9: 9 n + 2 (ny nz + nx nz + nx ny) floats of scratch (per-cell normal and
// ordered-pair shear stresses, and the shears one layer past the high faces);
// needs s.mu_c filled by launch_stress_coefficients
void launch_stress_diffuse(const StepView& s, float dt_sub, float* t9, float* const out[3], cudaStream_t st);
// needs s.mu_c filled by launch_stress_coefficients
void launch_viscosity_bound(const StepView& s, unsigned int* bound_bits, cudaStream_t st);
uint32_t fields_groups(const StepView& s);
// partials: 3 * fields_groups float4; scalars3: 3 float4 (the 12 diagnostics floats)
void launch_fields(const StepView& s, float4* cells, float4* partials, float4* scalars3, cudaStream_t st);

}  // namespace mhdproj
