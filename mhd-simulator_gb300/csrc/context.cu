// context.cu -- the C ABI of mhdproj.h: context lifetime, topology, the GB300
// solver's CG/refinement driver, the adjoint and the chained projection.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/mhdproj.h"
#include "kernels.h"
#include "reference.h"
#include "topology.h"

using namespace mhdproj;

static thread_local std::string g_create_error;
namespace mhdproj {
// Message for entry points that run without a context (read with
// mhdproj_last_error(NULL)).
void set_global_error(const std::string& msg) { g_create_error = msg; }
}  // namespace mhdproj

struct mhdproj_ctx {
    mhdproj_grid grid{};
    mhdproj_options opt{};
    std::string err;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    long long n = 0;
    long long nfx = 0, nfy = 0, nfz = 0;
    int outlet = 0;
    Launch L{};
    std::vector<void*> allocs;
    // topology and coefficients
    uint8_t* d_solid_prev = nullptr;
    uint8_t* d_cls = nullptr;
    int* d_flag = nullptr;
    int* h_flag = nullptr;
    // connected-component labels (u32 per cell), top-layer marks, counts
    uint32_t* d_labels = nullptr;
    uint32_t* d_roots = nullptr;
    uint8_t* d_topflag = nullptr;
    TopoCounts* d_topo = nullptr;
    TopoCounts* h_topo = nullptr;
    uint32_t components = 0, pinned = 0;
    // one component without an outlet: mean-free pressure, gauge at its root
    bool meanfree = false;
    long long root = -1;
    long long n_active = 0;
    bool have_topology = false, have_coef = false;
    float* alpha = nullptr;
    float4* coef = nullptr;
    void* coef_lo = nullptr;
    float* gtop = nullptr;
    float rho_l = 0.f, rho_air = 0.f;
    // thermal phase drag of the GB300 mobility (mhdproj_set_phase_drag)
    float* phase = nullptr;
    bool drag = false;
    float drag_rate = 0.f, drag_dt = 0.f;
    // solver state
    // double-FP32 pairs: right-hand side, potential, adjoint potential
    float *b_hi = nullptr, *b_lo = nullptr, *phi_hi = nullptr, *phi_lo = nullptr;
    float *psi_hi = nullptr, *psi_lo = nullptr;
    float *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *e = nullptr, *ztmp = nullptr;
    Scalars* sc = nullptr;
    Scalars* h_sc = nullptr;
    double* partials = nullptr;
    MGPlan mg{};
    bool use_mg = false;
    bool staged = true;  // finest-level stencils through shared-memory staging
    // pipelined CG: search+SpMV, fused V-cycle passes; ping-pong r and p
    bool pipelined = false;
    float *r1 = nullptr, *p1 = nullptr;
    uint64_t launches = 0;        // kernels launched (measurement)
    uint64_t graph_kernels = 0;   // kernels per replay of it_graph
    cudaGraphExec_t it_graph = nullptr;
    bool graph_failed = false;
    cudaEvent_t ev_a = nullptr, ev_b = nullptr, ev_sync = nullptr;
    bool have_solution = false;
    // host-buffer staging
    float *s_alpha = nullptr, *s_u = nullptr, *s_v = nullptr, *s_w = nullptr, *s_p = nullptr;
    uint8_t* s_solid = nullptr;
    // copy streams of the host-buffer path (created with its staging buffers)
    cudaStream_t cp[2] = {nullptr, nullptr};
    cudaEvent_t cp_ev[3] = {nullptr, nullptr, nullptr};
    // chain
    float *c_cur[3] = {nullptr, nullptr, nullptr}, *c_star[3] = {nullptr, nullptr, nullptr};
    float *c_lam[3] = {nullptr, nullptr, nullptr}, *c_lam2[3] = {nullptr, nullptr, nullptr};
    double* c_grad[3] = {nullptr, nullptr, nullptr};
    std::vector<float*> c_checkpoints;
    int c_steps = 0, c_every = 0;
    float c_dt = 0.f;
    bool c_ready = false;
    // objective 1 (summed over the chain's states): the force and a working
    // state kept for the backward pass, and the states of one checkpoint
    // segment recomputed there
    int c_objective = 0;
    float *c_force[3] = {nullptr, nullptr, nullptr}, *c_work[3] = {nullptr, nullptr, nullptr};
    std::vector<float*> c_segment;
    // fluid step and fields: rollback copies, predicted and viscous velocity,
    // reduction partials, and the last fields pass's CFL inputs
    float *st_prev[3] = {nullptr, nullptr, nullptr}, *st_pred[3] = {nullptr, nullptr, nullptr};
    float *st_star[3] = {nullptr, nullptr, nullptr}, *st_prev_p = nullptr;
    uint8_t* st_open[3] = {nullptr, nullptr, nullptr};
    float4* st_partials = nullptr;
    float4* st_scalars = nullptr;
    float4* h_st_scalars = nullptr;
    bool have_fields = false;
    bool step_ran = false;  // the step buffers hold a step's velocities (profiling)
    // moving-interface stress workspace (allocated by the first such step)
    float* st_mu = nullptr;
    float4 *st_t4 = nullptr, *st_y0 = nullptr, *st_f0 = nullptr;
    float2* st_t2 = nullptr;
    float* st_t9 = nullptr;
    unsigned int* st_bound = nullptr;
    float step_dt = 0.f, step_nu = 0.f;
    float max_face_speed = 0.f, force_max = 0.f;
    long long n_fluid = 0;
    // reference solver
    RefState* ref = nullptr;
};

static int fail(mhdproj_ctx* c, int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    else g_create_error = buf;
    return code;
}
#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t _e = (call);                                                                   \
        if (_e != cudaSuccess)                                                                     \
            return fail(ctx, _e == cudaErrorMemoryAllocation ? MHDPROJ_ERR_OUT_OF_MEMORY : MHDPROJ_ERR_CUDA, \
                        "%s: %s", #call, cudaGetErrorString(_e));                                  \
    } while (0)

template <class T>
static cudaError_t dalloc(mhdproj_ctx* ctx, T** p, size_t bytes) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, bytes ? bytes : 16);
    if (e != cudaSuccess) return e;
    ctx->allocs.push_back(q);
    *p = (T*)q;
    return cudaMemsetAsync(q, 0, bytes ? bytes : 16, ctx->stream);
}

static Fields fields(mhdproj_ctx* c) {
    Fields F{};
    F.cls = c->d_cls;
    F.alpha = c->alpha;
    F.coef = c->coef;
    F.coef_lo = c->coef_lo;
    F.coef_lo_kind = c->opt.precision;
    F.gtop = c->gtop;
    F.b_hi = c->b_hi;
    F.b_lo = c->b_lo;
    F.r = c->r;
    F.z = c->z;
    F.p = c->p;
    F.q = c->q;
    F.e = c->e;
    F.sc = c->sc;
    F.partials = c->partials;
    F.outlet = c->outlet;
    F.h = c->grid.h;
    F.rho_l = c->rho_l;
    F.rho_air = c->rho_air;
    F.mob.rho_l = c->rho_l;
    F.mob.rho_air = c->rho_air;
    F.mob.single = c->opt.two_phase == 0;
    F.mob.phase = c->drag ? c->phase : nullptr;
    F.mob.drag_rate = c->drag_rate;
    F.mob.dt = c->drag_dt;
    F.n_active = c->n_active;
    return F;
}

// Bounded host wait on the context stream (no unbounded spin).
static int wait_stream(mhdproj_ctx* ctx, double timeout_s = 600.0) {
    CK(cudaEventRecord(ctx->ev_sync, ctx->stream));
    auto t0 = std::chrono::steady_clock::now();
    int spins = 0;
    for (;;) {
        cudaError_t e = cudaEventQuery(ctx->ev_sync);
        if (e == cudaSuccess) return 0;
        if (e != cudaErrorNotReady) return fail(ctx, MHDPROJ_ERR_CUDA, "stream wait: %s", cudaGetErrorString(e));
        if (++spins > 2000) std::this_thread::sleep_for(std::chrono::microseconds(50));
        else std::this_thread::yield();
        double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (el > timeout_s) return fail(ctx, MHDPROJ_ERR_TIMEOUT, "device work did not finish within %.0f s", timeout_s);
    }
}
static int read_scalars(mhdproj_ctx* ctx) {
    CK(cudaMemcpyAsync(ctx->h_sc, ctx->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, ctx->stream));
    const int rc = wait_stream(ctx);
    if (rc == 0 && ctx->h_sc->stalled)
        return fail(ctx, MHDPROJ_ERR_TIMEOUT, "a bounded wait for staged data inside a smoothing pass expired");
    return rc;
}

// ------------------------------------------------------------ options
extern "C" void mhdproj_default_options(mhdproj_options* o) {
    memset(o, 0, sizeof *o);
    o->solver = MHDPROJ_SOLVER_GB300;
    o->precision = MHDPROJ_PRECISION_FP16;
    o->preconditioner = MHDPROJ_PRECOND_AUTO;
    o->rel_tol = 1e-6f;
    o->abs_div_tol = 0.0f;
    o->max_iterations = 20000;
    o->max_refinements = 4;
    o->two_phase = 1;
    o->gauge = -1;
    o->compute_divergence = 0;
}

extern "C" const char* mhdproj_last_error(const mhdproj_ctx* ctx) {
    return ctx ? ctx->err.c_str() : g_create_error.c_str();
}

// ----------------------------------------------------------- hierarchy
static int build_levels(mhdproj_ctx* ctx) {
    MGPlan& P = ctx->mg;
    P.precision = ctx->opt.precision;
    P.sc = ctx->sc;
    P.prolong = 2.0f;
    P.pin_coarse = -1;
    P.staged = ctx->staged;
    int d[3] = {(int)ctx->grid.nx, (int)ctx->grid.ny, (int)ctx->grid.nz};
    const int per = (int)ctx->grid.periodic;
    const size_t vbytes = P.precision == 0 ? 4 : 2;
    P.nlevels = 0;
    for (;;) {
        MGLevel& L = P.lv[P.nlevels];
        L.L = tile_launch(d[0], d[1], d[2], per, MAX_REDUCE_BLOCKS);
        L.odd_periodic = false;
        for (int a = 0; a < 3; a++)
            if ((per & (1 << a)) && (d[a] & 1) && d[a] >= 3) L.odd_periodic = true;
        const long long n = (long long)d[0] * d[1] * d[2];
        if (P.nlevels == 0) {
            L.coef32 = ctx->coef;
            L.coef_lo = ctx->coef_lo;
            L.r = ctx->r;
            L.e = ctx->z;
            L.tmp = nullptr;
            if (L.odd_periodic) CK(dalloc(ctx, (float**)&L.tmp, n * 4));
        } else {
            CK(dalloc(ctx, &L.coef32, n * sizeof(float4)));
            L.coef_lo = nullptr;
            if (P.precision != 0) CK(dalloc(ctx, (uint2**)&L.coef_lo, n * sizeof(uint2)));
            CK(dalloc(ctx, (char**)&L.r, n * vbytes));
            CK(dalloc(ctx, (char**)&L.e, n * vbytes));
            L.tmp = nullptr;
            if (L.odd_periodic) CK(dalloc(ctx, (char**)&L.tmp, n * vbytes));
        }
        P.nlevels++;
        // Coarsen until every extent is at most 4 (the reference's own stop):
        // the coarsest operator (<= 64 cells) is inverted exactly once per
        // coefficient set.
        if (d[0] <= 4 && d[1] <= 4 && d[2] <= 4) break;
        if (P.nlevels >= 31) return fail(ctx, MHDPROJ_ERR_INVALID, "multigrid hierarchy too deep");
        for (int a = 0; a < 3; a++) d[a] = (d[a] + 1) / 2;
    }
    P.m = d[0] * d[1] * d[2];
    CK(dalloc(ctx, &P.ainv, (size_t)P.m * P.m * sizeof(float)));
    P.bottom_img = nullptr;
    mg_plan_bottom(P);
    if (P.bottom_from > 0) {
        CK(dalloc(ctx, (char**)&P.bottom_img, (size_t)P.bottom.img_floats * sizeof(float)));
        P.bottom.img = P.bottom_img;
    }
    // Levels run as fused pre-/post-smoothing passes: a prefix of the levels
    // that have a coarser level, an x extent divisible by 4 and even periodic
    // extents, above 4096 cells; smaller levels run in the bottom sub-cycle.
    P.fused_levels = 0;
    P.e0 = nullptr;
    if (ctx->pipelined && P.nlevels >= 2) {
        int F = 0;
        while (F < P.nlevels - 1) {
            const Grid3& g = P.lv[F].L.g;
            if (!fused_supported(g)) break;
            if (F > 0 && g.n() <= 4096) break;  // the bottom sub-cycle takes over
            F++;
        }
        if (F == 0) {
            ctx->pipelined = false;
        } else {
            P.fused_levels = F;
            CK(dalloc(ctx, &P.e0, (size_t)ctx->n * 4));
            const size_t rbytes = P.precision == 0 ? 16 : 8;
            for (int l = 0; l < F; l++) {
                CK(dalloc(ctx, (char**)&P.lv[l].sm, (size_t)P.lv[l].L.g.n() * rbytes));
                if (l > 0) CK(dalloc(ctx, (char**)&P.lv[l].eo, (size_t)P.lv[l].L.g.n() * vbytes));
                if (l > 0 && P.w_from > 0 && l >= P.w_from && l <= P.w_to) {
                    CK(dalloc(ctx, (char**)&P.lv[l].r2, (size_t)P.lv[l].L.g.n() * vbytes));
                    CK(dalloc(ctx, (char**)&P.lv[l].eo2, (size_t)P.lv[l].L.g.n() * vbytes));
                }
            }
        }
    } else {
        ctx->pipelined = false;
    }
    return 0;
}

// --------------------------------------------------------- create/destroy
extern "C" int mhdproj_create(const mhdproj_grid* grid, const mhdproj_options* options, mhdproj_ctx** out) {
    mhdproj_ctx* ctx = nullptr;
    if (!grid || !out) return fail(nullptr, MHDPROJ_ERR_INVALID, "grid and out must not be NULL");
    *out = nullptr;
    mhdproj_options o;
    if (options) o = *options;
    else mhdproj_default_options(&o);
    const long long n = (long long)grid->nx * grid->ny * grid->nz;
    if (grid->nx == 0 || grid->ny == 0 || grid->nz == 0) return fail(nullptr, MHDPROJ_ERR_INVALID, "Invalid pressure grid dimensions");
    if (n >= (1ll << 31) - 1 || (long long)(grid->nx + 1) * grid->ny * grid->nz >= (1ll << 31) ||
        (long long)grid->nx * grid->ny * (grid->nz + 1) >= (1ll << 31))
        return fail(nullptr, MHDPROJ_ERR_INVALID, "Fluid allocation exceeds 32-bit cell indexing");
    if (!(grid->h > 0.0f) || !std::isfinite(grid->h)) return fail(nullptr, MHDPROJ_ERR_INVALID, "cell size must be positive");
    if (grid->boundary != MHDPROJ_BOUNDARY_REFERENCE_CLOSED && grid->boundary != MHDPROJ_BOUNDARY_OUTLET_TOP)
        return fail(nullptr, MHDPROJ_ERR_INVALID, "unknown boundary mode");
    if (grid->boundary == MHDPROJ_BOUNDARY_OUTLET_TOP && (grid->periodic & 4u))
        return fail(nullptr, MHDPROJ_ERR_INVALID, "a top outlet needs a non-periodic z axis");
    if (o.solver != MHDPROJ_SOLVER_REFERENCE && o.solver != MHDPROJ_SOLVER_GB300)
        return fail(nullptr, MHDPROJ_ERR_INVALID, "unknown solver");
    if (o.precision < 0 || o.precision > 2) return fail(nullptr, MHDPROJ_ERR_INVALID, "unknown precision");
    // FluidConfig::validate (src/fluid/mod.rs:56-80) limits; the GB300 solver
    // also accepts tolerances below 1e-7 because it refines in FP64.
    if (!std::isfinite(o.abs_div_tol) || o.abs_div_tol < 0.f || o.max_iterations < 1 || o.max_iterations > 1000000)
        return fail(nullptr, MHDPROJ_ERR_INVALID, "Invalid fluid timestep, initial condition or solver limits/tolerances");
    if (o.solver == MHDPROJ_SOLVER_REFERENCE) {
        if (!(o.rel_tol >= 1e-7f && o.rel_tol <= 1e-2f) || o.max_iterations > 20000)
            return fail(nullptr, MHDPROJ_ERR_INVALID, "Invalid fluid timestep, initial condition or solver limits/tolerances");
        if (grid->boundary != MHDPROJ_BOUNDARY_REFERENCE_CLOSED)
            return fail(nullptr, MHDPROJ_ERR_INVALID, "the reference solver has closed boundaries only");
    } else {
        if (!(o.rel_tol >= 1e-12f && o.rel_tol <= 1e-2f))
            return fail(nullptr, MHDPROJ_ERR_INVALID, "relative tolerance must lie in [1e-12, 1e-2]");
        if (o.max_refinements < 1 || o.max_refinements > 64)
            return fail(nullptr, MHDPROJ_ERR_INVALID, "max_refinements must lie in [1, 64]");
    }
    ctx = new mhdproj_ctx();
    ctx->grid = *grid;
    ctx->opt = o;
    ctx->n = n;
    ctx->nfx = (long long)(grid->nx + 1) * grid->ny * grid->nz;
    ctx->nfy = (long long)grid->nx * (grid->ny + 1) * grid->nz;
    ctx->nfz = (long long)grid->nx * grid->ny * (grid->nz + 1);
    ctx->outlet = grid->boundary == MHDPROJ_BOUNDARY_OUTLET_TOP;
    int rc = 0;
    auto bad = [&](int code) {
        g_create_error = ctx->err;
        mhdproj_destroy(ctx);
        return code;
    };
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        fail(ctx, MHDPROJ_ERR_CUDA, "cudaStreamCreate failed (is a GPU visible?)");
        return bad(MHDPROJ_ERR_CUDA);
    }
    ctx->own_stream = true;
    if (cudaEventCreate(&ctx->ev_a) != cudaSuccess || cudaEventCreate(&ctx->ev_b) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_sync, cudaEventDisableTiming) != cudaSuccess) {
        fail(ctx, MHDPROJ_ERR_CUDA, "cudaEventCreate failed");
        return bad(MHDPROJ_ERR_CUDA);
    }
    if (cudaMallocHost(&ctx->h_sc, sizeof(Scalars)) != cudaSuccess || cudaMallocHost(&ctx->h_flag, sizeof(int)) != cudaSuccess ||
        cudaMallocHost(&ctx->h_topo, sizeof(TopoCounts)) != cudaSuccess ||
        cudaMallocHost(&ctx->h_st_scalars, 3 * sizeof(float4)) != cudaSuccess) {
        fail(ctx, MHDPROJ_ERR_CUDA, "cudaMallocHost failed");
        return bad(MHDPROJ_ERR_CUDA);
    }
    // Per-cell kernels: short z runs in many blocks, so the last wave of
    // resident blocks is a small share of the launch.
    ctx->L = tile_launch(grid->nx, grid->ny, grid->nz, grid->periodic, MAX_REDUCE_BLOCKS);
    if ((rc = [&]() -> int {
             CK(dalloc(ctx, &ctx->d_solid_prev, n));
             CK(dalloc(ctx, &ctx->d_cls, n));
             CK(dalloc(ctx, &ctx->d_flag, sizeof(int)));
             CK(dalloc(ctx, &ctx->d_labels, n * 4));
             CK(dalloc(ctx, &ctx->d_roots, (n + 1) / 2 * 4));
             CK(dalloc(ctx, &ctx->d_topo, sizeof(TopoCounts)));
             if (ctx->outlet && !(grid->periodic & 4)) CK(dalloc(ctx, &ctx->d_topflag, n));
             CK(dalloc(ctx, &ctx->sc, sizeof(Scalars)));
             CK(dalloc(ctx, &ctx->partials, sizeof(double) * 4 * MAX_REDUCE_BLOCKS));
             if (ctx->opt.solver == MHDPROJ_SOLVER_REFERENCE) {
                 int r = ref_create(&ctx->ref, grid, &ctx->opt, ctx->stream, ctx->err);
                 return r;
             }
             CK(dalloc(ctx, &ctx->alpha, n * 4));
             CK(dalloc(ctx, &ctx->coef, n * sizeof(float4)));
             if (ctx->opt.precision != 0) CK(dalloc(ctx, (uint2**)&ctx->coef_lo, n * sizeof(uint2)));
             CK(dalloc(ctx, &ctx->gtop, (size_t)grid->nx * grid->ny * 4));
             CK(dalloc(ctx, &ctx->b_hi, n * 4));
             CK(dalloc(ctx, &ctx->b_lo, n * 4));
             CK(dalloc(ctx, &ctx->phi_hi, n * 4));
             CK(dalloc(ctx, &ctx->phi_lo, n * 4));
             CK(dalloc(ctx, &ctx->psi_hi, n * 4));
             CK(dalloc(ctx, &ctx->psi_lo, n * 4));
             CK(dalloc(ctx, &ctx->r, n * 4));
             CK(dalloc(ctx, &ctx->z, n * 4));
             CK(dalloc(ctx, &ctx->p, n * 4));
             CK(dalloc(ctx, &ctx->q, n * 4));
             CK(dalloc(ctx, &ctx->e, n * 4));
             ctx->use_mg = ctx->opt.preconditioner != MHDPROJ_PRECOND_JACOBI;
             {
                 const char* ev = getenv("MHDPROJ_STAGED");
                 if (ev && ev[0] == '0') ctx->staged = false;
                 if (!staged_supported(ctx->L.g)) ctx->staged = false;
                 const char* pv = getenv("MHDPROJ_PIPELINED");
                 ctx->pipelined = ctx->use_mg && ctx->staged && fused_supported(ctx->L.g) && !(pv && pv[0] == '0');
             }
             CK(staged_prepare_attributes());
             if (ctx->pipelined) {
                 CK(fused_prepare_attributes());
                 CK(dalloc(ctx, &ctx->r1, n * 4));
                 CK(dalloc(ctx, &ctx->p1, n * 4));
             }
             if (ctx->use_mg) {
                 int r = build_levels(ctx);
                 if (r) return r;
                 CK(mg_prepare_attributes());
             }
             CK(cudaStreamSynchronize(ctx->stream));
             return 0;
         }()) != 0)
        return bad(rc);
    *out = ctx;
    return 0;
}

extern "C" void mhdproj_destroy(mhdproj_ctx* ctx) {
    if (!ctx) return;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->it_graph) cudaGraphExecDestroy(ctx->it_graph);
    if (ctx->ref) ref_destroy(ctx->ref);
    for (void* p : ctx->allocs) cudaFree(p);
    for (float* p : ctx->c_checkpoints) cudaFree(p);
    for (float* p : ctx->c_segment) cudaFree(p);
    if (ctx->h_sc) cudaFreeHost(ctx->h_sc);
    if (ctx->h_flag) cudaFreeHost(ctx->h_flag);
    if (ctx->h_topo) cudaFreeHost(ctx->h_topo);
    for (cudaStream_t c : ctx->cp)
        if (c) cudaStreamDestroy(c);
    for (cudaEvent_t e : ctx->cp_ev)
        if (e) cudaEventDestroy(e);
    if (ctx->h_st_scalars) cudaFreeHost(ctx->h_st_scalars);
    if (ctx->ev_a) cudaEventDestroy(ctx->ev_a);
    if (ctx->ev_b) cudaEventDestroy(ctx->ev_b);
    if (ctx->ev_sync) cudaEventDestroy(ctx->ev_sync);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

extern "C" int mhdproj_set_stream(mhdproj_ctx* ctx, void* stream) {
    if (!ctx) return MHDPROJ_ERR_INVALID;
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    ctx->own_stream = false;
    ctx->stream = (cudaStream_t)stream;
    if (ctx->ref) ref_set_stream(ctx->ref, ctx->stream);
    return 0;
}

// -------------------------------------------------------- coefficients
__global__ void k_compare_u8(const uint8_t* a, const uint8_t* b, long long n, int* flag) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    int diff = 0;
    for (; i < n; i += stride) diff |= ((a[i] != 0) != (b[i] != 0));
    if (__syncthreads_or(diff) && threadIdx.x == 0) atomicOr(flag, 1);
}

// Mean-free gauge: the single gauge cell (class 2) becomes an active cell;
// its index is recorded.
__global__ void k_unpin(uint8_t* cls, long long n, int* root) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        if (cls[i] == 2) {
            cls[i] = 1;
            *root = (int)i;
        }
}

static int update_topology(mhdproj_ctx* ctx, const uint8_t* solid, bool* changed) {
    *changed = !ctx->have_topology;
    if (ctx->have_topology) {
        CK(cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream));
        k_compare_u8<<<152 * 4, 256, 0, ctx->stream>>>(solid, ctx->d_solid_prev, ctx->n, ctx->d_flag);
        ctx->launches += 1;
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(ctx->h_flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        int rc = wait_stream(ctx);
        if (rc) return rc;
        *changed = *ctx->h_flag != 0;
    }
    if (!*changed) return 0;
    CK(cudaMemcpyAsync(ctx->d_solid_prev, solid, ctx->n, cudaMemcpyDeviceToDevice, ctx->stream));
    // Components, gauge cells and counts on the GPU; only the counts come back.
    uint32_t* mask = ctx->ref ? ref_mask(ctx->ref) : nullptr;
    ctx->launches += (uint64_t)launch_topology(solid, (int)ctx->grid.nx, (int)ctx->grid.ny, (int)ctx->grid.nz,
                                               (int)ctx->grid.periodic, ctx->ref ? 0 : ctx->outlet, ctx->d_labels,
                                               ctx->d_roots, ctx->d_topflag, mask, ctx->ref ? nullptr : ctx->d_cls,
                                               ctx->d_topo, ctx->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(ctx->h_topo, ctx->d_topo, sizeof(TopoCounts), cudaMemcpyDeviceToHost, ctx->stream));
    int rc = wait_stream(ctx);
    if (rc) return rc;
    const TopoCounts t = *ctx->h_topo;
    if (t.error) {
        ctx->have_topology = false;
        return fail(ctx, MHDPROJ_ERR_CUDA, "connected-component labelling exceeded its step bound");
    }
    ctx->components = (uint32_t)t.components;
    ctx->n_fluid = (long long)t.fluid;
    if (ctx->ref) {
        ctx->n_active = (long long)t.fluid;
        ref_set_topology_device(ctx->ref, ctx->components, (uint32_t)t.fluid);
    } else {
        ctx->pinned = (uint32_t)t.pinned;
        ctx->meanfree = false;
        ctx->root = -1;
        ctx->mg.pin_coarse = -1;
        // One component that needs a gauge: mean-free pressure, as
        // configure_pressure_projection chooses for one connected component
        // (src/fluid/mod.rs:978-1002).  The operator is singular with the
        // constant null space; its root cell (the reference's anchor) fixes
        // the gauge of the result, and the coarsest multigrid solve pins the
        // coarsest cell that holds it.  A single pinned cell would leave a
        // near-null mode of eigenvalue ~1/N that FP16/BF16 level rounding
        // cannot resolve.
        if (t.components == 1 && t.pinned == 1 && ctx->opt.gauge != 0) {
            k_unpin<<<152 * 4, 256, 0, ctx->stream>>>(ctx->d_cls, ctx->n, ctx->d_flag);
            ctx->launches += 1;
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(ctx->h_flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
            rc = wait_stream(ctx);
            if (rc) return rc;
            ctx->meanfree = true;
            ctx->pinned = 0;
            ctx->root = *ctx->h_flag;
            if (ctx->use_mg) {
                const int L = ctx->mg.nlevels - 1;
                const long long nx = ctx->grid.nx, ny = ctx->grid.ny;
                const long long x = ctx->root % nx, y = (ctx->root / nx) % ny, z = ctx->root / (nx * ny);
                const Grid3& c = ctx->mg.lv[L].L.g;
                ctx->mg.pin_coarse = (int)((x >> L) + c.nx * ((y >> L) + c.ny * (z >> L)));
            }
        }
        ctx->n_active = (long long)(t.fluid - ctx->pinned);
    }
    ctx->have_topology = true;
    return 0;
}

static int rebuild_coefficients(mhdproj_ctx* ctx);

extern "C" int mhdproj_set_coefficients(mhdproj_ctx* ctx, const float* alpha, const uint8_t* solid, float rho_liquid,
                                        float rho_air) {
    if (!ctx || !alpha || !solid) return ctx ? fail(ctx, MHDPROJ_ERR_INVALID, "alpha and solid must not be NULL") : MHDPROJ_ERR_INVALID;
    if (!(rho_liquid > 0.f) || !std::isfinite(rho_liquid) || !(rho_air > 0.f) || !std::isfinite(rho_air))
        return fail(ctx, MHDPROJ_ERR_INVALID, "Fluid material needs a positive density");
    bool changed = false;
    int rc = update_topology(ctx, solid, &changed);
    if (rc) return rc;
    ctx->rho_l = rho_liquid;
    ctx->rho_air = rho_air;
    if (ctx->ref) {
        rc = ref_set_coefficients(ctx->ref, alpha, rho_liquid, rho_air, ctx->err);
        if (rc) return rc;
        ctx->have_coef = true;
        return 0;
    }
    CK(cudaMemcpyAsync(ctx->alpha, alpha, ctx->n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    return rebuild_coefficients(ctx);
}

// GB300 solver: the coefficient cache, smoother records and multigrid
// hierarchy from the stored liquid fraction, densities and phase drag.
static int rebuild_coefficients(mhdproj_ctx* ctx) {
    Fields F = fields(ctx);
    launch_coefficients(ctx->L, F, ctx->stream);
    ctx->launches += 1;
    CK(cudaGetLastError());
    if (ctx->use_mg) {
        mg_build(ctx->mg, ctx->stream);
        // Galerkin levels, the coarsest inverse and the bottom sub-cycle's image
        ctx->launches += (uint64_t)ctx->mg.nlevels + (ctx->mg.bottom_from > 0 && ctx->mg.bottom_img ? 1 : 0);
        if (ctx->pipelined) {
            mg_smoother_records(ctx->mg, ctx->stream);
            ctx->launches += (uint64_t)ctx->mg.fused_levels;
        }
        CK(cudaGetLastError());
    }
    ctx->have_coef = true;
    return 0;
}

extern "C" int mhdproj_set_phase_drag(mhdproj_ctx* ctx, const float* phase, float drag_rate, float dt) {
    if (!ctx) return MHDPROJ_ERR_INVALID;
    if (ctx->ref) return ref_set_phase_drag(ctx->ref, phase, drag_rate, dt, ctx->err);
    if (!phase) {
        ctx->drag = false;
    } else {
        if (!(drag_rate > 0.0f) || !(dt > 0.0f) || !std::isfinite(drag_rate) || !std::isfinite(dt))
            return fail(ctx, MHDPROJ_ERR_INVALID, "Invalid fluid timestep, initial condition or solver limits/tolerances");
        if (!ctx->phase) CK(dalloc(ctx, &ctx->phase, ctx->n * 4));
        CK(cudaMemcpyAsync(ctx->phase, phase, ctx->n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
        ctx->drag = true;
        ctx->drag_rate = drag_rate;
        ctx->drag_dt = dt;
    }
    // the mobility changed: rebuild the cache if coefficients are set
    return ctx->have_coef ? rebuild_coefficients(ctx) : 0;
}

// ------------------------------------------------------------- solver
__global__ void k_jacobi(Grid3 g, const float4* __restrict__ coef, const float* __restrict__ r, float* __restrict__ z,
                         const Scalars* sc) {
    if (sc->converged) return;
    const int x = blockIdx.x * TX + threadIdx.x, y = blockIdx.y * TY + threadIdx.y;
    if (x >= g.nx || y >= g.ny) return;
    const int z0 = blockIdx.z * g.zper, z1 = min(g.nz, z0 + g.zper);
    for (int zz = z0; zz < z1; zz++) {
        const int i = x + g.nx * (y + g.ny * zz);
        const float4 c = coef[i];
        float d = c.x + c.y + c.z + c.w;
        int xp = x + 1 < g.nx ? i + 1 : ((g.periodic & 1) ? i + 1 - g.nx : -1);
        int yp = y + 1 < g.ny ? i + g.nx : ((g.periodic & 2) ? i + g.nx - g.nx * g.ny : -1);
        int zp = zz + 1 < g.nz ? i + g.nx * g.ny : ((g.periodic & 4) ? i + g.nx * g.ny - g.nx * g.ny * g.nz : -1);
        if (xp >= 0) d += coef[xp].x;
        if (yp >= 0) d += coef[yp].y;
        if (zp >= 0) d += coef[zp].z;
        z[i] = d > 0.f ? sc->sigma * r[i] / d : 0.f;
    }
}
// Kernel counts of the enqueue paths (the launch counter of the context).
static uint64_t kernels_vcycle_from(const MGPlan& P, int from) {
    const int lb = (P.bottom_from > 0 && P.bottom_from >= from) ? P.bottom_from : P.nlevels;
    uint64_t k = 1;  // coarsest solve or the bottom sub-cycle
    for (int l = from; l + 1 < P.nlevels && l < lb; l++) {
        const uint64_t copy = P.lv[l].odd_periodic ? 1 : 0;
        k += 2 + copy + 1;      // red from zero, black (+ copy), restriction
        k += 1 + 2 + 2 * copy;  // prolongation, black, red (+ copies)
    }
    return k;
}
static uint64_t kernels_fused_solve(const MGPlan& P, int l) {
    if (l >= P.fused_levels) return kernels_vcycle_from(P, l);
    const uint64_t visit = 2 + kernels_fused_solve(P, l + 1);  // pre, coarser levels, post
    if (P.w_from > 0 && l >= P.w_from && l <= P.w_to) return 2 * visit + 1;  // + the second visit's residual
    return visit;
}
static uint64_t kernels_precondition(const mhdproj_ctx* ctx) {
    if (!ctx->use_mg) return 1;
    if (ctx->pipelined) return 2 + kernels_fused_solve(ctx->mg, 1);
    return kernels_vcycle_from(ctx->mg, 0);
}
static uint64_t kernels_iteration(const mhdproj_ctx* ctx) {
    if (ctx->pipelined) return 1 + kernels_precondition(ctx);  // search+SpMV, V-cycle passes
    return 4 + kernels_precondition(ctx);                       // SpMV, update, V-cycle, dot, search
}
static uint64_t kernels_pass_start(const mhdproj_ctx* ctx) {
    return kernels_precondition(ctx) + (ctx->pipelined ? 0 : 1);
}

static void enqueue_precondition(mhdproj_ctx* ctx) {
    if (ctx->use_mg) mg_vcycle(ctx->mg, ctx->stream);
    else k_jacobi<<<ctx->L.grid, ctx->L.block, 0, ctx->stream>>>(ctx->L.g, ctx->coef, ctx->r, ctx->z, ctx->sc);
}
// Pass start of the pipelined CG: z = B r0 and rz (the first search step
// then takes p = z).
static void enqueue_pass_start(mhdproj_ctx* ctx) {
    if (ctx->pipelined) {
        mg_vcycle_fused(ctx->mg, ctx->r, nullptr, nullptr, false, ctx->partials, ctx->n_active, ctx->stream);
        return;
    }
    enqueue_precondition(ctx);
    Fields F = fields(ctx);
    launch_dot_rz(ctx->L, F, 1, ctx->stream);
}
// Two pipelined CG iterations with the r and p buffers swapping roles.
static void enqueue_pipelined_pair(mhdproj_ctx* ctx) {
    float* rb[2] = {ctx->r, ctx->r1};
    float* pb[2] = {ctx->p, ctx->p1};
    for (int par = 0; par < 2; par++) {
        launch_search_spmv(ctx->L, ctx->coef, ctx->z, pb[par], pb[1 - par], ctx->e, ctx->q, ctx->sc, ctx->partials,
                           1 - par, ctx->stream);
        mg_vcycle_fused(ctx->mg, rb[par], ctx->q, rb[1 - par], true, ctx->partials, ctx->n_active, ctx->stream);
    }
}
static void enqueue_iteration_body(mhdproj_ctx* ctx) {
    if (ctx->pipelined) {
        enqueue_pipelined_pair(ctx);
        return;
    }
    Fields F = fields(ctx);
    if (ctx->staged) launch_spmv_staged(ctx->L, F, ctx->stream);
    else launch_spmv_pq(ctx->L, F, ctx->stream);
    launch_update(ctx->L, F, ctx->stream);
    enqueue_precondition(ctx);
    launch_dot_rz(ctx->L, F, 0, ctx->stream);
    launch_search(ctx->L, F, ctx->stream);
}

static int launch_iterations(mhdproj_ctx* ctx, int count) {
    if (!ctx->it_graph && !ctx->graph_failed) {
        cudaGraph_t graph = nullptr;
        CK(cudaStreamSynchronize(ctx->stream));
        cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            enqueue_iteration_body(ctx);
            e = cudaStreamEndCapture(ctx->stream, &graph);
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&ctx->it_graph, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            ctx->graph_failed = true;
            ctx->it_graph = nullptr;
        }
    }
    // a pipelined graph holds two iterations
    const int launches = ctx->pipelined ? (count + 1) / 2 : count;
    const uint64_t body = kernels_iteration(ctx) * (ctx->pipelined ? 2 : 1);
    for (int k = 0; k < launches; k++) {
        if (ctx->it_graph) CK(cudaGraphLaunch(ctx->it_graph, ctx->stream));
        else enqueue_iteration_body(ctx);
        ctx->launches += body;
    }
    CK(cudaGetLastError());
    return 0;
}

// Solve A x = b (the double-FP32 pair in ctx->b_hi/b_lo, ||b||^2 in sc->bb)
// by CG with iterative refinement: each pass solves A e = r in FP32 and adds
// e to the double-FP32 solution x, whose residual b - A x is recomputed in
// double-FP32.  x holds the initial guess.  Returns 0 or an error.
static int solve(mhdproj_ctx* ctx, float* x_hi, float* x_lo, mhdproj_stats* st, bool x_zero = false) {
    Fields F = fields(ctx);
    const double tol2 = (double)ctx->opt.rel_tol * ctx->opt.rel_tol;
    (void)tol2;
    int passes = 0;
    // x_zero: the right-hand-side kernel already set up the first pass (r = b)
    if (!x_zero) launch_residual(ctx->L, F, x_hi, x_lo, ctx->stream);
    enqueue_pass_start(ctx);
    ctx->launches += (x_zero ? 0 : 1) + kernels_pass_start(ctx);
    CK(cudaGetLastError());
    int rc = read_scalars(ctx);
    if (rc) return rc;
    const uint32_t max_it = ctx->opt.max_iterations;
    for (;;) {
        Scalars& S = *ctx->h_sc;
        if (S.nonfinite) return fail(ctx, MHDPROJ_ERR_NONFINITE, "Nonfinite fluid pressure residual");
        if (S.outer_done) break;
        if (passes > ctx->opt.max_refinements || (uint32_t)S.total_iterations >= max_it) {
            const double rel = S.bb > 0 ? std::sqrt(S.rr_true / S.bb) : 0.0;
            const double floor_ = ctx->opt.abs_div_tol;
            return fail(ctx, MHDPROJ_ERR_NOT_CONVERGED,
                        "Fluid pressure solve did not converge after %d iterations (true relative residual %.3e, "
                        "requested %.3e, RMS divergence floor %.3e s\xe2\x81\xbb\xc2\xb9)",
                        S.total_iterations, rel, (double)ctx->opt.rel_tol, floor_);
        }
        // inner CG on A e = r
        int batch = 4;
        double rr_prev = S.rr;
        int it_prev = S.iterations;
        while (!ctx->h_sc->converged && (uint32_t)ctx->h_sc->total_iterations < max_it) {
            int room = (int)(max_it - (uint32_t)ctx->h_sc->total_iterations);
            int b = std::min(batch, room);
            rc = launch_iterations(ctx, b);
            if (rc) return rc;
            rc = read_scalars(ctx);
            if (rc) return rc;
            Scalars& T = *ctx->h_sc;
            if (T.nonfinite) return fail(ctx, MHDPROJ_ERR_NONFINITE, "Nonfinite fluid pressure residual");
            if (T.converged) break;
            if (T.iterations <= it_prev) return fail(ctx, MHDPROJ_ERR_NO_PROGRESS, "Fluid pressure iteration made no progress");
            // predict the remaining iterations from the observed contraction
            const int done = T.iterations - it_prev;
            double rate = (rr_prev > 0 && T.rr > 0) ? std::pow(T.rr / rr_prev, 1.0 / done) : 0.5;
            int need = 16;
            if (rate > 0 && rate < 1 && T.rr > T.rr_target) need = (int)std::ceil(std::log(T.rr_target / T.rr) / std::log(rate));
            batch = std::max(1, std::min(16, need));
            rr_prev = T.rr;
            it_prev = T.iterations;
        }
        if (ctx->pipelined) launch_accumulate_pipelined(ctx->L, x_hi, x_lo, ctx->e, ctx->p, ctx->p1, ctx->sc, ctx->stream);
        else launch_accumulate(ctx->L, F, x_hi, x_lo, ctx->stream);
        if (ctx->h_sc->breakdown && ctx->use_mg && ctx->mg.w_from > 0) {
            // The W-cycle step lost positive definiteness on this operator:
            // V-cycles from here on (the iteration graph is recaptured), and
            // the pass does not count against the refinement limit.
            ctx->mg.w_disabled = true;
            mg_plan_bottom(ctx->mg);
            if (ctx->it_graph) {
                cudaGraphExecDestroy(ctx->it_graph);
                ctx->it_graph = nullptr;
            }
            CK(cudaMemsetAsync(reinterpret_cast<char*>(ctx->sc) + offsetof(Scalars, breakdown), 0, sizeof(int),
                               ctx->stream));
        } else {
            passes++;
        }
        launch_residual(ctx->L, F, x_hi, x_lo, ctx->stream);
        enqueue_pass_start(ctx);
        ctx->launches += 2 + kernels_pass_start(ctx);  // accumulate, residual, pass start
        CK(cudaGetLastError());
        rc = read_scalars(ctx);
        if (rc) return rc;
    }
    if (st) {
        const Scalars& S = *ctx->h_sc;
        st->iterations = (uint32_t)S.total_iterations;
        st->refinements = (uint32_t)(passes > 0 ? passes - 1 : 0);
        st->true_relative_residual = S.bb > 0 ? std::sqrt(S.rr_true / S.bb) : 0.0;
        st->relative_residual = (float)st->true_relative_residual;
        st->multigrid = ctx->use_mg;
        st->levels = ctx->use_mg ? (uint32_t)ctx->mg.nlevels : 0;
        long long cc = 0;
        if (ctx->use_mg)
            for (int l = 1; l < ctx->mg.nlevels; l++) cc += ctx->mg.lv[l].L.g.n();
        st->coarse_cells = (uint64_t)cc;
    }
    return 0;
}

static void begin_scalars(mhdproj_ctx* ctx) {
    const double tol2 = (double)ctx->opt.rel_tol * ctx->opt.rel_tol;
    const double h = ctx->grid.h;
    const double abs_floor = (double)ctx->opt.abs_div_tol * ctx->opt.abs_div_tol * h * h * h * h * (double)ctx->n_active;
    // FP32 CG reduces its own residual by about 1e-5 reliably; refine beyond.
    launch_init_scalars(ctx->sc, tol2, abs_floor, 1e-10, (int)ctx->opt.max_iterations, ctx->stream);
}

static const char* const MEANFREE_ADJOINT =
    "the adjoint needs an outlet or pinned gauges; this domain is one closed component (mean-free pressure): "
    "create the context with mhdproj_options.gauge = 0";

// The phase-drag mobility depends on dt; a call with another dt is refused
// (the reference rebuilds its coefficients with the step's dt).
static int check_drag_dt(mhdproj_ctx* ctx, float dt) {
    if (ctx->drag && dt != ctx->drag_dt)
        return fail(ctx, MHDPROJ_ERR_INVALID,
                    "the phase-drag mobility was set for a different dt; call mhdproj_set_phase_drag again");
    return 0;
}

// Mean-free gauge: the potential is defined up to a constant; take the one
// that is zero at the root cell (the reference's pressure of the mean-free
// mode, p = rho_l (phi - phi_anchor) / dt, src/fluid/solver.wgsl:269-270).
// The root itself is left alone while the others read it, then zeroed.
__global__ void k_shift_gauge(Grid3 g, const uint8_t* __restrict__ cls, float* __restrict__ hi,
                              float* __restrict__ lo, long long root) {
    const df pr = {hi[root], lo[root]};
    const long long n = g.n();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        if (i == root || cls[i] == 0) continue;
        const df d = df_sub(df{hi[i], lo[i]}, pr);
        hi[i] = d.hi;
        lo[i] = d.lo;
    }
}
static int shift_gauge(mhdproj_ctx* ctx) {
    k_shift_gauge<<<152 * 8, 256, 0, ctx->stream>>>(ctx->L.g, ctx->d_cls, ctx->phi_hi, ctx->phi_lo, ctx->root);
    ctx->launches += 1;
    CK(cudaGetLastError());
    CK(cudaMemsetAsync(ctx->phi_hi + ctx->root, 0, sizeof(float), ctx->stream));
    CK(cudaMemsetAsync(ctx->phi_lo + ctx->root, 0, sizeof(float), ctx->stream));
    return 0;
}

static int project_gb300(mhdproj_ctx* ctx, const float* us, const float* vs, const float* ws, float* uo, float* vo,
                         float* wo, float* po, float dt, int warm, mhdproj_stats* st) {
    if (!ctx->have_coef) return fail(ctx, MHDPROJ_ERR_STATE, "call mhdproj_set_coefficients before projecting");
    if (int rc = check_drag_dt(ctx, dt)) return rc;
    CK(cudaEventRecord(ctx->ev_a, ctx->stream));
    begin_scalars(ctx);
    Fields F = fields(ctx);
    const bool from_zero = !warm || !ctx->have_solution;
    launch_rhs(ctx->L, F, us, vs, ws, ctx->stream, from_zero);
    ctx->launches += 2;
    if (from_zero) {
        CK(cudaMemsetAsync(ctx->phi_hi, 0, ctx->n * 4, ctx->stream));
        CK(cudaMemsetAsync(ctx->phi_lo, 0, ctx->n * 4, ctx->stream));
    }
    mhdproj_stats local{};
    int rc = solve(ctx, ctx->phi_hi, ctx->phi_lo, &local, from_zero);
    if (rc) return rc;
    if (ctx->meanfree) {
        rc = shift_gauge(ctx);
        if (rc) return rc;
    }
    launch_correct(ctx->L, F, ctx->phi_hi, ctx->phi_lo, us, vs, ws, uo, vo, wo, po, dt, ctx->stream);
    ctx->launches += 1;
    if (ctx->opt.compute_divergence) {
        launch_divergence(ctx->L, F, uo, vo, wo, ctx->stream);
        ctx->launches += 1;
    }
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev_b, ctx->stream));
    if (ctx->opt.compute_divergence) {
        rc = read_scalars(ctx);
        if (rc) return rc;
        local.max_divergence = ctx->h_sc->divmax;
        local.rms_divergence = ctx->n_active ? std::sqrt(ctx->h_sc->div2 / (double)ctx->n_active) : 0.0;
    } else {
        rc = wait_stream(ctx);
        if (rc) return rc;
    }
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ctx->ev_a, ctx->ev_b));
    local.elapsed_ms = ms;
    local.meanfree = 0;
    ctx->have_solution = true;
    if (st) *st = local;
    return 0;
}

extern "C" int mhdproj_project(mhdproj_ctx* ctx, const float* usx, const float* usy, const float* usz, float* uox,
                               float* uoy, float* uoz, float* p_out, float dt, int warm_start, mhdproj_stats* stats) {
    if (!ctx) return MHDPROJ_ERR_INVALID;
    if (!usx || !usy || !usz || !uox || !uoy || !uoz) return fail(ctx, MHDPROJ_ERR_INVALID, "face arrays must not be NULL");
    if (!(dt > 0.f) || !std::isfinite(dt)) return fail(ctx, MHDPROJ_ERR_INVALID, "Invalid fluid timestep, initial condition or solver limits/tolerances");
    if (ctx->ref) {
        if (!ctx->have_coef) return fail(ctx, MHDPROJ_ERR_STATE, "call mhdproj_set_coefficients before projecting");
        mhdproj_stats local{};
        CK(cudaEventRecord(ctx->ev_a, ctx->stream));
        int rc = ref_project(ctx->ref, usx, usy, usz, uox, uoy, uoz, p_out, dt, warm_start, &local, ctx->err);
        if (rc) return rc;
        CK(cudaEventRecord(ctx->ev_b, ctx->stream));
        rc = wait_stream(ctx);
        if (rc) return rc;
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, ctx->ev_a, ctx->ev_b));
        local.elapsed_ms = ms;
        if (stats) *stats = local;
        return 0;
    }
    return project_gb300(ctx, usx, usy, usz, uox, uoy, uoz, p_out, dt, warm_start, stats);
}

extern "C" int mhdproj_project_host(mhdproj_ctx* ctx, const float* alpha, const uint8_t* solid, float rho_liquid,
                                    float rho_air, const float* usx, const float* usy, const float* usz, float* uox,
                                    float* uoy, float* uoz, float* p_out, float dt, int warm_start,
                                    mhdproj_stats* stats) {
    if (!ctx) return MHDPROJ_ERR_INVALID;
    if (!alpha || !solid || !usx || !usy || !usz || !uox || !uoy || !uoz)
        return fail(ctx, MHDPROJ_ERR_INVALID, "host arrays must not be NULL");
    if (!ctx->s_alpha) {
        CK(dalloc(ctx, &ctx->s_alpha, ctx->n * 4));
        CK(dalloc(ctx, &ctx->s_solid, ctx->n));
        CK(dalloc(ctx, &ctx->s_u, ctx->nfx * 4));
        CK(dalloc(ctx, &ctx->s_v, ctx->nfy * 4));
        CK(dalloc(ctx, &ctx->s_w, ctx->nfz * 4));
        CK(dalloc(ctx, &ctx->s_p, ctx->n * 4));
    }
    if (!ctx->cp[0]) {
        for (int k = 0; k < 2; k++) CK(cudaStreamCreateWithFlags(&ctx->cp[k], cudaStreamNonBlocking));
        for (int k = 0; k < 3; k++) CK(cudaEventCreateWithFlags(&ctx->cp_ev[k], cudaEventDisableTiming));
    }
    // The copies run on three streams (the context's and two copy streams),
    // each array in three slices, so several copy engines share the link;
    // the face velocities arrive while the coefficients are being built.
    cudaStream_t s = ctx->stream;
    cudaStream_t st3[3] = {s, ctx->cp[0], ctx->cp[1]};
    auto spread = [&](void* dst, const void* src, size_t bytes, cudaMemcpyKind kind) -> int {
        const size_t slice = (bytes / 3 + 255) & ~(size_t)255;
        for (int k = 0; k < 3; k++) {
            const size_t off = std::min(bytes, slice * (size_t)k), end = std::min(bytes, slice * (size_t)(k + 1));
            if (end > off)
                CK(cudaMemcpyAsync((char*)dst + off, (const char*)src + off, end - off, kind, st3[k]));
        }
        return 0;
    };
    // the copy streams start after the context stream's earlier work
    CK(cudaEventRecord(ctx->cp_ev[0], s));
    for (int k = 0; k < 2; k++) CK(cudaStreamWaitEvent(ctx->cp[k], ctx->cp_ev[0], 0));
    int rc = spread(ctx->s_alpha, alpha, ctx->n * 4, cudaMemcpyHostToDevice);
    if (!rc) rc = spread(ctx->s_solid, solid, ctx->n, cudaMemcpyHostToDevice);
    if (rc) return rc;
    for (int k = 0; k < 2; k++) {
        CK(cudaEventRecord(ctx->cp_ev[1 + k], ctx->cp[k]));
        CK(cudaStreamWaitEvent(s, ctx->cp_ev[1 + k], 0));  // alpha and solid complete on the context stream
    }
    // face velocities on the copy streams, behind the coefficient set-up
    CK(cudaMemcpyAsync(ctx->s_u, usx, ctx->nfx * 4, cudaMemcpyHostToDevice, ctx->cp[0]));
    CK(cudaMemcpyAsync(ctx->s_v, usy, ctx->nfy * 4, cudaMemcpyHostToDevice, ctx->cp[1]));
    CK(cudaMemcpyAsync(ctx->s_w, usz, ctx->nfz * 4, cudaMemcpyHostToDevice, ctx->cp[0]));
    rc = mhdproj_set_coefficients(ctx, ctx->s_alpha, ctx->s_solid, rho_liquid, rho_air);
    if (rc) return rc;
    for (int k = 0; k < 2; k++) {
        CK(cudaEventRecord(ctx->cp_ev[1 + k], ctx->cp[k]));
        CK(cudaStreamWaitEvent(s, ctx->cp_ev[1 + k], 0));
    }
    rc = mhdproj_project(ctx, ctx->s_u, ctx->s_v, ctx->s_w, ctx->s_u, ctx->s_v, ctx->s_w, ctx->s_p, dt, warm_start,
                         stats);
    if (rc) return rc;
    CK(cudaEventRecord(ctx->cp_ev[0], s));
    for (int k = 0; k < 2; k++) CK(cudaStreamWaitEvent(ctx->cp[k], ctx->cp_ev[0], 0));
    rc = spread(uox, ctx->s_u, ctx->nfx * 4, cudaMemcpyDeviceToHost);
    if (!rc) rc = spread(uoy, ctx->s_v, ctx->nfy * 4, cudaMemcpyDeviceToHost);
    if (!rc) rc = spread(uoz, ctx->s_w, ctx->nfz * 4, cudaMemcpyDeviceToHost);
    if (!rc && p_out) rc = spread(p_out, ctx->s_p, ctx->n * 4, cudaMemcpyDeviceToHost);
    if (rc) return rc;
    for (int k = 0; k < 2; k++) {
        CK(cudaEventRecord(ctx->cp_ev[1 + k], ctx->cp[k]));
        CK(cudaStreamWaitEvent(s, ctx->cp_ev[1 + k], 0));
    }
    return wait_stream(ctx);
}

// -------------------------------------------------------------- adjoint
static int vjp_gb300(mhdproj_ctx* ctx, const float* gu, const float* gv, const float* gw, const float* gp, float dt,
                     float* ou, float* ov, float* ow, mhdproj_stats* st) {
    begin_scalars(ctx);
    Fields F = fields(ctx);
    launch_adj_rhs(ctx->L, F, gu, gv, gw, gp, dt, ctx->stream);
    ctx->launches += 2;
    CK(cudaMemsetAsync(ctx->psi_hi, 0, ctx->n * 4, ctx->stream));
    CK(cudaMemsetAsync(ctx->psi_lo, 0, ctx->n * 4, ctx->stream));
    int rc = solve(ctx, ctx->psi_hi, ctx->psi_lo, st);
    if (rc) return rc;
    launch_adj_correct(ctx->L, F, ctx->psi_hi, ctx->psi_lo, gu, gv, gw, ou, ov, ow, ctx->stream);
    ctx->launches += 1;
    CK(cudaGetLastError());
    return 0;
}

extern "C" int mhdproj_project_vjp(mhdproj_ctx* ctx, const float* gux, const float* guy, const float* guz,
                                   const float* gp, float dt, float* ogx, float* ogy, float* ogz,
                                   mhdproj_stats* stats) {
    if (!ctx) return MHDPROJ_ERR_INVALID;
    if (ctx->ref) return fail(ctx, MHDPROJ_ERR_INVALID, "the adjoint is part of the GB300 solver");
    if (!ctx->have_coef) return fail(ctx, MHDPROJ_ERR_STATE, "call mhdproj_set_coefficients before the adjoint");
    if (!gux || !guy || !guz || !ogx || !ogy || !ogz) return fail(ctx, MHDPROJ_ERR_INVALID, "face arrays must not be NULL");
    if (!(dt > 0.f)) return fail(ctx, MHDPROJ_ERR_INVALID, "dt must be positive");
    if (int rc = check_drag_dt(ctx, dt)) return rc;
    if (ctx->meanfree) return fail(ctx, MHDPROJ_ERR_INVALID, MEANFREE_ADJOINT);
    CK(cudaEventRecord(ctx->ev_a, ctx->stream));
    mhdproj_stats local{};
    int rc = vjp_gb300(ctx, gux, guy, guz, gp, dt, ogx, ogy, ogz, &local);
    if (rc) return rc;
    CK(cudaEventRecord(ctx->ev_b, ctx->stream));
    rc = wait_stream(ctx);
    if (rc) return rc;
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ctx->ev_a, ctx->ev_b));
    local.elapsed_ms = ms;
    if (stats) *stats = local;
    return 0;
}

// ---------------------------------------------------------------- chain
__global__ void k_d2f(const double* a, float* b, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

static int chain_alloc(mhdproj_ctx* ctx) {
    if (ctx->c_ready) return 0;
    const long long m[3] = {ctx->nfx, ctx->nfy, ctx->nfz};
    for (int a = 0; a < 3; a++) {
        CK(dalloc(ctx, &ctx->c_cur[a], m[a] * 4));
        CK(dalloc(ctx, &ctx->c_star[a], m[a] * 4));
        CK(dalloc(ctx, &ctx->c_lam[a], m[a] * 4));
        CK(dalloc(ctx, &ctx->c_lam2[a], m[a] * 4));
        CK(dalloc(ctx, &ctx->c_grad[a], m[a] * 8));
    }
    ctx->c_ready = true;
    return 0;
}

// One chain step on the state `cur` in place: u* = u + dt f / rho_face into
// c_star, then the projection of u* back into `cur`.
static int chain_step(mhdproj_ctx* ctx, float* const cur[3], const float* fx, const float* fy, const float* fz,
                      float dt, mhdproj_stats* total) {
    cudaStream_t s = ctx->stream;
    Fields F = fields(ctx);
    launch_add_force(ctx->L, F, cur[0], cur[1], cur[2], fx, fy, fz, dt, ctx->c_star[0], ctx->c_star[1],
                     ctx->c_star[2], s);
    mhdproj_stats one{};
    begin_scalars(ctx);
    launch_rhs(ctx->L, F, ctx->c_star[0], ctx->c_star[1], ctx->c_star[2], s);
    CK(cudaMemsetAsync(ctx->phi_hi, 0, ctx->n * 4, s));
    CK(cudaMemsetAsync(ctx->phi_lo, 0, ctx->n * 4, s));
    int rc = solve(ctx, ctx->phi_hi, ctx->phi_lo, &one);
    if (rc) return rc;
    launch_correct(ctx->L, F, ctx->phi_hi, ctx->phi_lo, ctx->c_star[0], ctx->c_star[1], ctx->c_star[2], cur[0], cur[1],
                   cur[2], nullptr, dt, s);
    total->iterations += one.iterations;
    total->refinements += one.refinements;
    total->true_relative_residual = std::max(total->true_relative_residual, one.true_relative_residual);
    return 0;
}

extern "C" int mhdproj_chain_set_objective(mhdproj_ctx* ctx, int kind) {
    if (!ctx) return MHDPROJ_ERR_INVALID;
    if (ctx->ref) return fail(ctx, MHDPROJ_ERR_INVALID, "the chained adjoint is part of the GB300 solver");
    if (kind != MHDPROJ_CHAIN_FINAL_OUTLET && kind != MHDPROJ_CHAIN_SUMMED_OUTLET)
        return fail(ctx, MHDPROJ_ERR_INVALID, "unknown chain objective (0: final outlet plane, 1: summed over the steps)");
    ctx->c_objective = kind;
    ctx->c_steps = 0;  // a chain run under the other objective is not differentiated
    return 0;
}

extern "C" int mhdproj_chain_forward(mhdproj_ctx* ctx, const float* u0x, const float* u0y, const float* u0z,
                                     const float* fx, const float* fy, const float* fz, float dt, int steps,
                                     int checkpoint_every, float* ufx, float* ufy, float* ufz, double* objective,
                                     mhdproj_stats* stats) {
    if (!ctx) return MHDPROJ_ERR_INVALID;
    if (ctx->ref) return fail(ctx, MHDPROJ_ERR_INVALID, "the chained adjoint is part of the GB300 solver");
    if (!ctx->have_coef) return fail(ctx, MHDPROJ_ERR_STATE, "call mhdproj_set_coefficients before the chain");
    if (steps < 1 || checkpoint_every < 1 || !(dt > 0.f)) return fail(ctx, MHDPROJ_ERR_INVALID, "steps, checkpoint_every and dt must be positive");
    if (int rc = check_drag_dt(ctx, dt)) return rc;
    if (ctx->meanfree) return fail(ctx, MHDPROJ_ERR_INVALID, MEANFREE_ADJOINT);
    int rc = chain_alloc(ctx);
    if (rc) return rc;
    ctx->c_steps = 0;  // differentiable again once this chain has finished
    const long long m[3] = {ctx->nfx, ctx->nfy, ctx->nfz};
    const float* u0[3] = {u0x, u0y, u0z};
    cudaStream_t s = ctx->stream;
    for (int a = 0; a < 3; a++) CK(cudaMemcpyAsync(ctx->c_cur[a], u0[a], m[a] * 4, cudaMemcpyDeviceToDevice, s));
    // checkpoints: the state entering every checkpoint_every-th step
    const int nck = (steps + checkpoint_every - 1) / checkpoint_every;
    while ((int)ctx->c_checkpoints.size() < 3 * nck) {
        float* p = nullptr;
        const int a = (int)ctx->c_checkpoints.size() % 3;
        CK(cudaMalloc(&p, m[a] * 4));
        ctx->c_checkpoints.push_back(p);
    }
    const bool summed = ctx->c_objective == MHDPROJ_CHAIN_SUMMED_OUTLET;
    if (summed) {
        // the backward pass recomputes states from the checkpoints with this force
        for (int a = 0; a < 3; a++)
            if (!ctx->c_force[a]) {
                CK(dalloc(ctx, &ctx->c_force[a], m[a] * 4));
                CK(dalloc(ctx, &ctx->c_work[a], m[a] * 4));
            }
        const float* f[3] = {fx, fy, fz};
        for (int a = 0; a < 3; a++) CK(cudaMemcpyAsync(ctx->c_force[a], f[a], m[a] * 4, cudaMemcpyDeviceToDevice, s));
        CK(cudaMemsetAsync(reinterpret_cast<char*>(ctx->sc) + offsetof(Scalars, objective), 0, sizeof(double), s));
    }
    CK(cudaEventRecord(ctx->ev_a, s));
    Fields F = fields(ctx);
    mhdproj_stats total{};
    for (int k = 0; k < steps; k++) {
        if (k % checkpoint_every == 0) {
            const int c = k / checkpoint_every;
            for (int a = 0; a < 3; a++)
                CK(cudaMemcpyAsync(ctx->c_checkpoints[3 * c + a], ctx->c_cur[a], m[a] * 4, cudaMemcpyDeviceToDevice, s));
        }
        rc = chain_step(ctx, ctx->c_cur, fx, fy, fz, dt, &total);
        if (rc) return rc;
        // objective 1: the outlet term of every state after a step
        if (summed) launch_outlet_objective(ctx->L, F, ctx->c_cur[2], nullptr, s, true);
    }
    if (!summed) launch_outlet_objective(ctx->L, F, ctx->c_cur[2], nullptr, s);
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev_b, s));
    rc = read_scalars(ctx);
    if (rc) return rc;
    if (objective) *objective = ctx->h_sc->objective;
    const float* cur[3] = {ctx->c_cur[0], ctx->c_cur[1], ctx->c_cur[2]};
    float* uf[3] = {ufx, ufy, ufz};
    for (int a = 0; a < 3; a++)
        if (uf[a]) CK(cudaMemcpyAsync(uf[a], cur[a], m[a] * 4, cudaMemcpyDeviceToDevice, s));
    rc = wait_stream(ctx);
    if (rc) return rc;
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ctx->ev_a, ctx->ev_b));
    total.elapsed_ms = ms;
    total.relative_residual = (float)total.true_relative_residual;
    ctx->c_steps = steps;
    ctx->c_every = checkpoint_every;
    ctx->c_dt = dt;
    if (stats) *stats = total;
    return 0;
}

extern "C" int mhdproj_chain_backward(mhdproj_ctx* ctx, float* gfx, float* gfy, float* gfz, mhdproj_stats* stats) {
    if (!ctx) return MHDPROJ_ERR_INVALID;
    if (!ctx->c_ready || ctx->c_steps < 1) return fail(ctx, MHDPROJ_ERR_STATE, "run mhdproj_chain_forward first");
    if (!gfx || !gfy || !gfz) return fail(ctx, MHDPROJ_ERR_INVALID, "gradient arrays must not be NULL");
    const long long m[3] = {ctx->nfx, ctx->nfy, ctx->nfz};
    cudaStream_t s = ctx->stream;
    CK(cudaEventRecord(ctx->ev_a, s));
    // lambda_K = dJ/du_K: 2 w on the outlet faces of the final state, 0 elsewhere
    for (int a = 0; a < 3; a++) {
        CK(cudaMemsetAsync(ctx->c_lam[a], 0, m[a] * 4, s));
        CK(cudaMemsetAsync(ctx->c_grad[a], 0, m[a] * 8, s));
    }
    if (ctx->outlet) launch_outlet_objective(ctx->L, fields(ctx), ctx->c_cur[2], ctx->c_lam[2], s);
    Fields F = fields(ctx);
    mhdproj_stats total{};
    float* lam[3] = {ctx->c_lam[0], ctx->c_lam[1], ctx->c_lam[2]};
    float* nxt[3] = {ctx->c_lam2[0], ctx->c_lam2[1], ctx->c_lam2[2]};
    // lambda <- P^T lambda (the VJP of step k's projection) and dJ/df +=
    // dt / rho_face times it
    auto adjoint_step = [&]() -> int {
        mhdproj_stats one{};
        int rc = vjp_gb300(ctx, lam[0], lam[1], lam[2], nullptr, ctx->c_dt, nxt[0], nxt[1], nxt[2], &one);
        if (rc) return rc;
        launch_force_grad(ctx->L, F, nxt[0], nxt[1], nxt[2], ctx->c_dt, ctx->c_grad[0], ctx->c_grad[1], ctx->c_grad[2], s);
        std::swap(lam[0], nxt[0]);
        std::swap(lam[1], nxt[1]);
        std::swap(lam[2], nxt[2]);
        total.iterations += one.iterations;
        total.refinements += one.refinements;
        total.true_relative_residual = std::max(total.true_relative_residual, one.true_relative_residual);
        return 0;
    };
    if (ctx->c_objective != MHDPROJ_CHAIN_SUMMED_OUTLET) {
        // J depends on the final state only: the adjoint steps need no
        // forward state (the projection's VJP does not depend on it)
        for (int k = ctx->c_steps - 1; k >= 0; k--)
            if (int rc = adjoint_step()) return rc;
    } else {
        // J sums the outlet term of every state u_1 .. u_K, so step k's
        // adjoint adds 2 w_k on the outlet faces: the states of each
        // checkpoint segment are recomputed from its checkpoint (at most
        // checkpoint_every - 1 forward steps per segment), last segment first
        const int K = ctx->c_steps, every = ctx->c_every;
        const int nck = (K + every - 1) / every;
        while ((int)ctx->c_segment.size() < 3 * (every - 1)) {
            float* p = nullptr;
            const int a = (int)ctx->c_segment.size() % 3;
            CK(cudaMalloc(&p, m[a] * 4));
            ctx->c_segment.push_back(p);
        }
        const float* fo[3] = {ctx->c_force[0], ctx->c_force[1], ctx->c_force[2]};
        for (int j = nck - 1; j >= 0; j--) {
            const int s0 = j * every, e0 = std::min(K, s0 + every);
            for (int a = 0; a < 3; a++)
                CK(cudaMemcpyAsync(ctx->c_work[a], ctx->c_checkpoints[3 * j + a], m[a] * 4, cudaMemcpyDeviceToDevice, s));
            for (int k = s0; k + 1 < e0; k++) {  // u_{k+1} into segment slot k - s0
                if (int rc = chain_step(ctx, ctx->c_work, fo[0], fo[1], fo[2], ctx->c_dt, &total)) return rc;
                for (int a = 0; a < 3; a++)
                    CK(cudaMemcpyAsync(ctx->c_segment[3 * (k - s0) + a], ctx->c_work[a], m[a] * 4,
                                       cudaMemcpyDeviceToDevice, s));
            }
            for (int k = e0 - 1; k >= s0; k--) {
                if (int rc = adjoint_step()) return rc;
                if (k >= 1 && ctx->outlet) {
                    const float* wk = k == s0 ? ctx->c_checkpoints[3 * j + 2] : ctx->c_segment[3 * (k - s0 - 1) + 2];
                    launch_outlet_objective(ctx->L, F, wk, lam[2], s, false, true);
                }
            }
        }
    }
    float* out[3] = {gfx, gfy, gfz};
    for (int a = 0; a < 3; a++) k_d2f<<<152 * 4, 256, 0, s>>>(ctx->c_grad[a], out[a], m[a]);
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev_b, s));
    int rc = wait_stream(ctx);
    if (rc) return rc;
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ctx->ev_a, ctx->ev_b));
    total.elapsed_ms = ms;
    total.relative_residual = (float)total.true_relative_residual;
    if (stats) *stats = total;
    return 0;
}

// --------------------------------------------------------------- probes
extern "C" int mhdproj_apply_operator(mhdproj_ctx* ctx, const float* x, float* y) {
    if (!ctx) return MHDPROJ_ERR_INVALID;
    if (!ctx->have_coef) return fail(ctx, MHDPROJ_ERR_STATE, "call mhdproj_set_coefficients first");
    if (ctx->ref) {
        int rc = ref_apply_operator(ctx->ref, x, y, ctx->err);
        if (rc) return rc;
        return wait_stream(ctx);
    }
    launch_apply(ctx->L, fields(ctx), x, y, ctx->stream);
    CK(cudaGetLastError());
    return wait_stream(ctx);
}

extern "C" int mhdproj_apply_preconditioner(mhdproj_ctx* ctx, const float* r, float* z) {
    if (!ctx) return MHDPROJ_ERR_INVALID;
    if (!ctx->have_coef) return fail(ctx, MHDPROJ_ERR_STATE, "call mhdproj_set_coefficients first");
    if (ctx->ref) {
        int rc = ref_apply_preconditioner(ctx->ref, r, z, ctx->err);
        if (rc) return rc;
        return wait_stream(ctx);
    }
    CK(cudaMemcpyAsync(ctx->r, r, ctx->n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    launch_set_sigma(ctx->sc, 1.0f, ctx->stream);
    enqueue_precondition(ctx);
    CK(cudaMemcpyAsync(z, ctx->z, ctx->n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaGetLastError());
    return wait_stream(ctx);
}

extern "C" int mhdproj_copy_coefficients(mhdproj_ctx* ctx, float* coef4) {
    if (!ctx) return MHDPROJ_ERR_INVALID;
    if (!ctx->have_coef) return fail(ctx, MHDPROJ_ERR_STATE, "call mhdproj_set_coefficients first");
    if (ctx->ref) {
        int rc = ref_copy_coefficients(ctx->ref, coef4, ctx->err);
        if (rc) return rc;
        return wait_stream(ctx);
    }
    CK(cudaMemcpyAsync(coef4, ctx->coef, ctx->n * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->stream));
    return wait_stream(ctx);
}

extern "C" int mhdproj_copy_potential(mhdproj_ctx* ctx, double* phi) {
    if (!ctx) return MHDPROJ_ERR_INVALID;
    if (ctx->ref) {
        int rc = ref_copy_potential(ctx->ref, phi, ctx->err);
        if (rc) return rc;
        return wait_stream(ctx);
    }
    launch_to_double(ctx->phi_hi, ctx->phi_lo, phi, ctx->n, ctx->stream);
    CK(cudaGetLastError());
    return wait_stream(ctx);
}

extern "C" int mhdproj_copy_topology(mhdproj_ctx* ctx, uint32_t* mask_host, uint32_t* components) {
    if (!ctx) return MHDPROJ_ERR_INVALID;
    if (!ctx->have_topology) return fail(ctx, MHDPROJ_ERR_STATE, "call mhdproj_set_coefficients first");
    if (mask_host) {
        if (ctx->ref) {
            CK(cudaMemcpyAsync(mask_host, ref_mask(ctx->ref), ctx->n * 4, cudaMemcpyDeviceToHost, ctx->stream));
        } else {
            std::vector<uint8_t> cls(ctx->n);
            CK(cudaMemcpyAsync(cls.data(), ctx->d_cls, ctx->n, cudaMemcpyDeviceToHost, ctx->stream));
            int rc = wait_stream(ctx);
            if (rc) return rc;
            for (long long i = 0; i < ctx->n; i++) mask_host[i] = cls[i];
        }
        int rc = wait_stream(ctx);
        if (rc) return rc;
    }
    if (components) *components = ctx->components;
    return 0;
}

// ----------------------------------------------------------- fluid step
static int step_buffers(mhdproj_ctx* ctx) {
    if (ctx->st_partials) return 0;
    const long long nf[3] = {ctx->nfx, ctx->nfy, ctx->nfz};
    for (int a = 0; a < 3; a++) {
        CK(dalloc(ctx, &ctx->st_prev[a], nf[a] * 4));
        CK(dalloc(ctx, &ctx->st_pred[a], nf[a] * 4));
        CK(dalloc(ctx, &ctx->st_star[a], nf[a] * 4));
        CK(dalloc(ctx, &ctx->st_open[a], nf[a]));
    }
    CK(dalloc(ctx, &ctx->st_prev_p, ctx->n * 4));
    CK(dalloc(ctx, &ctx->st_partials, (size_t)3 * ((ctx->n + 255) / 256) * sizeof(float4)));
    CK(dalloc(ctx, &ctx->st_scalars, 3 * sizeof(float4)));
    return 0;
}

// The fields of a velocity (u, v, w) with the context's potential.
static StepView step_view(mhdproj_ctx* ctx, const float* u, const float* v, const float* w, const float* em,
                          const float acc[3], float dt) {
    StepView sv{};
    sv.dims[0] = ctx->grid.nx;
    sv.dims[1] = ctx->grid.ny;
    sv.dims[2] = ctx->grid.nz;
    sv.dims[3] = (uint32_t)ctx->n;
    sv.periodic = ctx->grid.periodic;
    sv.h = ctx->grid.h;
    sv.dt = dt;
    for (int a = 0; a < 3; a++) sv.acc[a] = acc ? acc[a] : 0.0f;
    sv.vel[0] = u;
    sv.vel[1] = v;
    sv.vel[2] = w;
    sv.em = reinterpret_cast<const float4*>(em);
    if (ctx->ref) {
        const RefExport e = ref_export(ctx->ref);
        sv.mask = e.mask;
        sv.occ = e.occ;
        sv.phase = e.phase;
        sv.phi = e.work;
        sv.phi_stride = 4;
        sv.mean_free = e.mean_free;
        sv.two_phase = e.two_phase;
        sv.rho_l = e.rho_l;
        sv.rho_air = e.rho_air;
        sv.drag_rate = e.drag_rate;
    } else {
        sv.cls = ctx->d_cls;
        sv.occ = ctx->alpha;
        sv.phi = ctx->phi_hi;
        sv.phi_stride = 1;
        sv.two_phase = ctx->rho_air != ctx->rho_l;
        sv.rho_l = ctx->rho_l;
        sv.rho_air = ctx->rho_air;
        if (ctx->drag) {
            sv.phase = ctx->phase;
            sv.drag_rate = ctx->drag_rate;
        }
    }
    return sv;
}

// fields + diagnostics, then read_diagnostics (src/fluid/mod.rs:1116-1143).
// *bad: a field is non-finite or out of range.
static int run_fields(mhdproj_ctx* ctx, const StepView& sv, float* cells, mhdproj_diagnostics* d, bool* bad) {
    int rc = step_buffers(ctx);
    if (rc) return rc;
    launch_fields(sv, reinterpret_cast<float4*>(cells), ctx->st_partials, ctx->st_scalars, ctx->stream);
    ctx->launches += 2;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(ctx->h_st_scalars, ctx->st_scalars, 3 * sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream));
    rc = wait_stream(ctx);
    if (rc) return rc;
    const float* s = reinterpret_cast<const float*>(ctx->h_st_scalars);
    *bad = s[7] != 0.0f;
    for (int k = 0; k < 12; k++) *bad = *bad || !std::isfinite(s[k]);
    const long long fl = ctx->ref ? (long long)ref_export(ctx->ref).fluid_cells : ctx->n_fluid;
    const float h = ctx->grid.h, h3 = h * h * h;
    mhdproj_diagnostics out{};
    out.max_speed_m_s = s[0];
    out.max_divergence_s_inv = s[1];
    out.rms_divergence_s_inv = std::sqrt(s[2] / (float)(fl > 1 ? fl : 1));
    out.kinetic_energy_j = s[3];
    out.fluid_mass_kg = sv.rho_l * s[9] * h3;
    out.max_pressure_pa = s[4];
    out.net_flux_m3_s = s[5] * h3;
    out.max_force_density = s[6];
    out.max_face_speed_m_s = s[8];
    out.nonfinite_cells = std::isfinite(s[7]) && s[7] > 0.f ? (uint32_t)s[7] : 0u;
    if (d) *d = out;
    if (!*bad) {
        ctx->max_face_speed = s[8];
        ctx->force_max = s[6];
        ctx->have_fields = true;
    }
    return 0;
}

extern "C" int mhdproj_fields(mhdproj_ctx* ctx, const float* u, const float* v, const float* w, const float* em_force,
                              const float acceleration[3], float dt, float* cells, mhdproj_diagnostics* diagnostics) {
    if (!ctx) return MHDPROJ_ERR_INVALID;
    if (!u || !v || !w) return fail(ctx, MHDPROJ_ERR_INVALID, "face arrays must not be NULL");
    if (!ctx->have_coef) return fail(ctx, MHDPROJ_ERR_STATE, "call mhdproj_set_coefficients first");
    if (!(dt > 0.f) || !std::isfinite(dt))
        return fail(ctx, MHDPROJ_ERR_INVALID, "Invalid fluid timestep, initial condition or solver limits/tolerances");
    const StepView sv = step_view(ctx, u, v, w, em_force, acceleration, dt);
    bool bad = false;
    int rc = run_fields(ctx, sv, cells, diagnostics, &bad);
    if (rc) return rc;
    if (bad) return fail(ctx, MHDPROJ_ERR_NONFINITE, "Nonfinite fluid fields; state restored");
    return 0;
}

// Velocity (and pressure) back to their values on entry.
static int step_restore(mhdproj_ctx* ctx, float* const vel[3], float* p_out) {
    const long long nf[3] = {ctx->nfx, ctx->nfy, ctx->nfz};
    for (int a = 0; a < 3; a++)
        CK(cudaMemcpyAsync(vel[a], ctx->st_prev[a], nf[a] * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    if (p_out) CK(cudaMemcpyAsync(p_out, ctx->st_prev_p, ctx->n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    return wait_stream(ctx);
}

static int stress_buffers(mhdproj_ctx* ctx) {
    if (ctx->st_mu) return 0;
    CK(dalloc(ctx, &ctx->st_mu, ctx->n * 4));
    CK(dalloc(ctx, &ctx->st_t4, ctx->n * sizeof(float4)));
    CK(dalloc(ctx, &ctx->st_t2, ctx->n * sizeof(float2)));
    CK(dalloc(ctx, &ctx->st_y0, ctx->n * sizeof(float4)));
    CK(dalloc(ctx, &ctx->st_f0, ctx->n * sizeof(float4)));
    const long long ghosts = 2ll * ((long long)ctx->grid.ny * ctx->grid.nz + (long long)ctx->grid.nx * ctx->grid.nz +
                                    (long long)ctx->grid.nx * ctx->grid.ny);
    CK(dalloc(ctx, &ctx->st_t9, (ctx->n * 9 + ghosts) * sizeof(float)));
    CK(dalloc(ctx, &ctx->st_bound, sizeof(unsigned int)));
    return 0;
}

// stabilized::schedule (src/fluid/stabilized.rs:11-50): rows of the damped
// second-order Runge-Kutta-Chebyshev method (Verwer, Hundsdorfer & Sommeijer
// 1990) for `euler_steps` equivalent Euler steps of dt: mu, nu, 1 - mu - nu,
// operator time, initial-operator time (FP64 recurrences rounded to FP32).
static std::vector<std::array<float, 5>> rkc_schedule(double dt, uint32_t euler_steps) {
    const double damping = 0.05;
    const double stiffness = 1.8 * (double)euler_steps;
    const uint32_t cap = (uint32_t)std::ceil(3.0 * std::sqrt((double)euler_steps)) + 2u;
    std::vector<std::array<float, 5>> rows;
    for (uint32_t stages = 2; stages <= cap; stages++) {
        const double w0 = 1.0 + damping / ((double)stages * (double)stages);
        std::vector<double> t{1.0, w0}, d{0.0, 1.0}, dd{0.0, 0.0};
        for (uint32_t j = 2; j <= stages; j++) {
            t.push_back(2.0 * w0 * t[j - 1] - t[j - 2]);
            d.push_back(2.0 * t[j - 1] + 2.0 * w0 * d[j - 1] - d[j - 2]);
            dd.push_back(4.0 * d[j - 1] + 2.0 * w0 * dd[j - 1] - dd[j - 2]);
        }
        const double w1 = d[stages] / dd[stages];
        if (stiffness > 0.9 * (1.0 + w0) / w1) continue;
        std::vector<double> b(t.size(), 0.0);
        for (size_t j = 2; j < t.size(); j++) b[j] = dd[j] / (d[j] * d[j]);
        b[0] = b[2];
        b[1] = b[2];
        rows.push_back({1.0f, 0.0f, 0.0f, (float)(dt * b[1] * w1), 0.0f});
        for (uint32_t j = 2; j <= stages; j++) {
            const float mu = (float)(2.0 * w0 * b[j] / b[j - 1]);
            const float nu = (float)(-b[j] / b[j - 2]);
            const double op = dt * 2.0 * w1 * b[j] / b[j - 1];
            const double a = 1.0 - b[j - 1] * t[j - 1];
            rows.push_back({mu, nu, 1.0f - mu - nu, (float)op, (float)(-a * op)});
        }
        return rows;
    }
    return rows;
}

// FluidState::diffuse_surface_stress (src/fluid/mod.rs:1160-1240) on the
// predicted velocity in st_pred; st_prev holds the step's starting velocity
// (copied into st_star, the second RKC stage buffer).  *substeps: Euler
// substeps or RKC stages.
static int diffuse_surface_stress(mhdproj_ctx* ctx, StepView S, float dt, uint32_t max_substeps,
                                  uint32_t* substeps) {
    *substeps = 0;
    // global_viscous_bound (:1146-1159): valid for every accepted fraction
    // distribution, rounded upward
    const double liquid = S.rho_l, ambient = S.rho_air;
    const double slack = (double)1e-5f + 4.0 * (double)FLT_EPSILON;
    const double floor_rho = std::min(liquid, ambient) - std::fabs(liquid - ambient) * slack;
    const double mu = (double)std::max(S.nu * S.rho_l, S.mu_air);
    const double h = ctx->grid.h;
    double count = 0.0;
    const double host_bound = 24.0 * mu / (floor_rho * h * h) * (1.0 + 32.0 * (double)FLT_EPSILON);
    for (int a = 0; a < 3; a++) S.vel[a] = ctx->st_pred[a];
    if (floor_rho > 0.0 && (double)dt * host_bound <= 1.8) {
        if (host_bound == 0.0) return 0;
        count = 1.0;
    } else {
        CK(cudaMemsetAsync(ctx->st_bound, 0, sizeof(unsigned int), ctx->stream));
        launch_stress_coefficients(S, ctx->stream);
        launch_viscosity_bound(S, ctx->st_bound, ctx->stream);
        ctx->launches += 7;
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(ctx->h_st_scalars, ctx->st_bound, sizeof(unsigned int), cudaMemcpyDeviceToHost,
                           ctx->stream));
        int rc = wait_stream(ctx);
        if (rc) return rc;
        unsigned int bits;
        memcpy(&bits, ctx->h_st_scalars, sizeof bits);
        float bound;
        memcpy(&bound, &bits, sizeof bound);
        if (!std::isfinite(bound) || bound < 0.f)
            return fail(ctx, MHDPROJ_ERR_NONFINITE, "Nonfinite viscous stability bound");
        if (bound == 0.f) return 0;
        count = std::max(std::ceil((double)dt * (double)bound / 1.8), 1.0);
    }
    if (count > (double)max_substeps)
        return fail(ctx, MHDPROJ_ERR_INVALID,
                    "Viscosity requires %.0f equivalent Euler substeps, above the %u work limit; reduce the common "
                    "timestep or increase Viscosity work limit",
                    count, max_substeps);
    const uint32_t steps = (uint32_t)count;
    const long long nf[3] = {ctx->nfx, ctx->nfy, ctx->nfz};
    float* const P[3] = {ctx->st_pred[0], ctx->st_pred[1], ctx->st_pred[2]};
    float* const V[3] = {ctx->st_star[0], ctx->st_star[1], ctx->st_star[2]};
    auto copy3 = [&](float* const dst[3], float* const src[3]) -> int {
        for (int a = 0; a < 3; a++)
            CK(cudaMemcpyAsync(dst[a], src[a], nf[a] * 4, cudaMemcpyDeviceToDevice, ctx->stream));
        return 0;
    };
    if (steps > 8u) {
        const auto rows = rkc_schedule((double)dt, steps);
        int rc = copy3(V, ctx->st_prev);  // the stage before the first one: the starting velocity
        if (rc) return rc;
        for (int a = 0; a < 3; a++) S.vel[a] = P[a];
        launch_stress_coefficients(S, ctx->stream);
        launch_stress_tensor(S, ctx->stream);
        launch_stress_save_initial(S, ctx->stream);
        ctx->launches += 3;
        for (size_t i = 0; i < rows.size(); i++) {
            const bool odd = i % 2 == 1;
            for (int a = 0; a < 3; a++) S.vel[a] = odd ? V[a] : P[a];
            if (i > 0) {
                launch_stress_tensor(S, ctx->stream);
                ctx->launches += 1;
            }
            launch_stress_stage(S, rows[i].data(), odd ? P : V, ctx->stream);
            ctx->launches += 3;
        }
        CK(cudaGetLastError());
        if (rows.size() % 2 == 1) {
            rc = copy3(P, V);
            if (rc) return rc;
        }
        *substeps = (uint32_t)rows.size();
        return 0;
    }
    const float dt_sub = (float)((double)dt / (double)steps);
    launch_stress_coefficients(S, ctx->stream);  // the cell viscosity the stresses read
    ctx->launches += 1;
    for (uint32_t k = 0; k < steps; k++) {
        for (int a = 0; a < 3; a++) S.vel[a] = P[a];
        launch_stress_diffuse(S, dt_sub, ctx->st_t9, V, ctx->stream);
        ctx->launches += 6;
        int rc = copy3(P, V);
        if (rc) return rc;
    }
    CK(cudaGetLastError());
    *substeps = steps;
    return 0;
}

extern "C" int mhdproj_fluid_step(mhdproj_ctx* ctx, float* u, float* v, float* w, const float* em_force,
                                  const mhdproj_step_params* sp, float* p_out, float* cells, mhdproj_stats* stats,
                                  mhdproj_diagnostics* diagnostics) {
    if (!ctx) return MHDPROJ_ERR_INVALID;
    if (!u || !v || !w || !sp) return fail(ctx, MHDPROJ_ERR_INVALID, "face arrays and step parameters must not be NULL");
    if (!ctx->have_coef) return fail(ctx, MHDPROJ_ERR_STATE, "call mhdproj_set_coefficients first");
    const float dt = sp->dt;
    bool ok = dt > 0.f && std::isfinite(dt) && std::isfinite(sp->kinematic_viscosity) && sp->kinematic_viscosity >= 0.f;
    for (int a = 0; a < 3; a++) ok = ok && std::isfinite(sp->acceleration[a]);
    if (!ok) return fail(ctx, MHDPROJ_ERR_INVALID, "Invalid fluid timestep, initial condition or solver limits/tolerances");
    ok = std::isfinite(sp->surface_tension) && sp->surface_tension >= 0.f && std::isfinite(sp->air_viscosity) &&
         sp->air_viscosity >= 0.f;
    if (!ok) return fail(ctx, MHDPROJ_ERR_INVALID, "surface tension and air viscosity must be finite and >= 0");
    StepView base = step_view(ctx, u, v, w, em_force, sp->acceleration, dt);
    const bool surface = base.two_phase != 0;  // a moving interface: two densities
    base.nu = sp->kinematic_viscosity;
    base.sigma = sp->surface_tension;
    base.mu_air = sp->air_viscosity;
    base.curv = sp->curvature;
    const uint32_t max_substeps = sp->max_viscous_substeps ? sp->max_viscous_substeps : 4096u;
    if (ctx->ref && base.phase && dt != ref_export(ctx->ref).drag_dt)
        return fail(ctx, MHDPROJ_ERR_INVALID,
                    "the phase-drag mobility was set for a different dt; call mhdproj_set_phase_drag again");
    if (!ctx->ref) {
        if (int rc = check_drag_dt(ctx, dt)) return rc;
    }
    int rc = step_buffers(ctx);
    if (rc) return rc;
    float* const vel[3] = {u, v, w};
    // velocity CFL limit (src/fluid/mod.rs:1255-1262) on the last fields
    if (!ctx->have_fields) {
        bool bad = false;
        rc = run_fields(ctx, base, nullptr, nullptr, &bad);
        if (rc) return rc;
        if (bad) return fail(ctx, MHDPROJ_ERR_NONFINITE, "Nonfinite fluid fields; state restored");
    }
    {
        const float* g = sp->acceleration;
        const float acceleration = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]) + ctx->force_max / base.rho_l;
        if ((ctx->max_face_speed * std::sqrt(3.0f) + acceleration * dt) * dt / ctx->grid.h > 0.9f)
            return fail(ctx, MHDPROJ_ERR_INVALID, "Fluid timestep exceeds the velocity CFL limit; reduce Δt");
        if (surface) {  // :1263-1275
            const float h = ctx->grid.h, sigma = sp->surface_tension;
            const float pi = 3.14159265358979323846f;
            const float capillary =
                sigma > 0.f ? std::sqrt((base.rho_l + base.rho_air) * (h * h * h) / (2.f * pi * sigma)) : INFINITY;
            if (dt > capillary || 3.f * (ctx->max_face_speed + acceleration * dt) * dt / h > 0.45f)
                return fail(ctx, MHDPROJ_ERR_INVALID,
                            "Moving-interface capillary or conservative CFL limit exceeded; reduce common timestep");
        }
    }
    const long long nf[3] = {ctx->nfx, ctx->nfy, ctx->nfz};
    for (int a = 0; a < 3; a++)
        CK(cudaMemcpyAsync(ctx->st_prev[a], vel[a], nf[a] * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    if (p_out) CK(cudaMemcpyAsync(ctx->st_prev_p, p_out, ctx->n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    // predict (advection) and viscous (viscosity, forcing, mobility)
    StepView sv = base;
    // with a moving interface the interface transport carries the momentum
    sv.advection = !surface && sp->advection != 0;
    launch_predict(sv, ctx->st_pred, ctx->st_star, ctx->st_open, ctx->stream);
    ctx->launches += 6;
    uint32_t substeps = 0;
    if (surface) {
        rc = stress_buffers(ctx);
        if (rc) return rc;
        StepView ss = sv;
        ss.mu_c = ctx->st_mu;
        ss.t4 = ctx->st_t4;
        ss.t2 = ctx->st_t2;
        ss.y0 = ctx->st_y0;
        ss.f0 = ctx->st_f0;
        rc = diffuse_surface_stress(ctx, ss, dt, max_substeps, &substeps);
        if (rc) {
            const std::string msg = ctx->err;
            step_restore(ctx, vel, p_out);
            ctx->err = msg;
            return rc;
        }
    }
    for (int a = 0; a < 3; a++) {
        sv.vel[a] = ctx->st_pred[a];
        sv.open[a] = ctx->st_open[a];
    }
    launch_viscous(sv, ctx->st_star, ctx->stream);
    ctx->launches += 3;
    CK(cudaGetLastError());
    ctx->step_ran = true;
    ctx->step_dt = dt;
    ctx->step_nu = sp->kinematic_viscosity;
    // the warm-started projection of the viscous velocity into (u, v, w)
    rc = mhdproj_project(ctx, ctx->st_star[0], ctx->st_star[1], ctx->st_star[2], u, v, w, p_out, dt, 1, stats);
    if (rc) {
        const std::string msg = ctx->err;
        step_restore(ctx, vel, p_out);
        ctx->err = msg;
        return rc;
    }
    // fields and diagnostics of the projected velocity; the cell records are
    // written once the diagnostics accept the step
    StepView fv = step_view(ctx, u, v, w, em_force, sp->acceleration, dt);
    fv.curv = sp->curvature;
    bool bad = false;
    rc = run_fields(ctx, fv, nullptr, diagnostics, &bad);
    if (rc) return rc;
    if (diagnostics) diagnostics->viscous_substeps = substeps;
    if (bad) {
        step_restore(ctx, vel, p_out);
        return fail(ctx, MHDPROJ_ERR_NONFINITE, "Nonfinite fluid fields; state restored");
    }
    if (cells) {
        launch_fields(fv, reinterpret_cast<float4*>(cells), ctx->st_partials, ctx->st_scalars, ctx->stream);
        ctx->launches += 2;
        CK(cudaGetLastError());
        return wait_stream(ctx);
    }
    return 0;
}


// ---------------------------------------------------------- measurement
// One launch of profiled kernel `kind` (rep r) on stream s.
static void profile_launch(mhdproj_ctx* ctx, int kind, int r, const Fields& F, cudaStream_t s) {
    switch (kind) {
        case 0:
            if (ctx->staged) launch_spmv_staged(ctx->L, F, s);
            else launch_spmv_pq(ctx->L, F, s);
            break;
        case 1: launch_update(ctx->L, F, s); break;
        case 2: mg_fine_smooth(ctx->mg, r & 1, s); break;
        case 3: mg_fine_restrict(ctx->mg, s); break;
        case 4: mg_fine_prolong(ctx->mg, s); break;
        case 5: launch_dot_rz(ctx->L, F, 0, s); break;
        case 6: launch_search(ctx->L, F, s); break;
        case 7: launch_residual(ctx->L, F, ctx->phi_hi, ctx->phi_lo, s); break;
        case 8: launch_coefficients(ctx->L, F, s); break;
        case 9:
            // relabels the current mask: the same classes are rewritten
            launch_topology(ctx->d_solid_prev, (int)ctx->grid.nx, (int)ctx->grid.ny, (int)ctx->grid.nz,
                            (int)ctx->grid.periodic, ctx->outlet, ctx->d_labels, ctx->d_roots,
                            ctx->d_topflag, nullptr, ctx->d_cls, ctx->d_topo, s);
            break;
        case 20:
        case 21:
        case 22: {
            const float g[3] = {0.0f, 0.0f, -9.81f};
            StepView sv = step_view(ctx, ctx->st_prev[0], ctx->st_prev[1], ctx->st_prev[2], nullptr, g,
                                    ctx->step_dt);
            sv.advection = 1;
            sv.nu = ctx->step_nu;
            if (kind == 20) launch_predict(sv, ctx->st_pred, ctx->st_star, ctx->st_open, s);
            if (kind == 21) {
                for (int a = 0; a < 3; a++) {
                    sv.vel[a] = ctx->st_pred[a];
                    sv.open[a] = ctx->st_open[a];
                }
                launch_viscous(sv, ctx->st_star, s);
            }
            if (kind == 22) launch_fields(sv, nullptr, ctx->st_partials, ctx->st_scalars, s);
            break;
        }
        case 10:
            launch_search_spmv(ctx->L, ctx->coef, ctx->z, ctx->p, ctx->p1, ctx->e, ctx->q, ctx->sc,
                               ctx->partials, 1, s);
            break;
        case 11: mg_fused_pre(ctx->mg, ctx->r, ctx->q, ctx->r1, ctx->partials, s); break;
        case 12: mg_fused_post(ctx->mg, ctx->r1, ctx->partials, ctx->n_active, s); break;
        case 13: mg_fused_coarse(ctx->mg, ctx->partials, ctx->n_active, s); break;
        case 14: mg_bottom_cycle(ctx->mg, s); break;
    }
}

extern "C" int mhdproj_profile_kernels(mhdproj_ctx* ctx, int reps, mhdproj_kernel_time* out, int max_out, int* count) {
    if (!ctx || !out || !count) return MHDPROJ_ERR_INVALID;
    if (ctx->ref) return fail(ctx, MHDPROJ_ERR_INVALID, "kernel profiling covers the GB300 solver");
    if (!ctx->have_coef) return fail(ctx, MHDPROJ_ERR_STATE, "call mhdproj_set_coefficients first");
    if (reps < 1) reps = 1;
    cudaStream_t s = ctx->stream;
    Fields F = fields(ctx);
    const double n = (double)ctx->n;
    const double cb = ctx->opt.precision == 0 ? 16.0 : 8.0;  // smoother coefficient bytes per cell
    struct Item {
        const char* name;
        double bytes_per_cell;
        int per_it;
        int kind;
    };
    // Algorithmic bytes per cell: the compulsory traffic of each kernel's
    // fields, every field touched once per launch.
    const double vbc = ctx->opt.precision == 0 ? 4.0 : 2.0;   // level-1 vector bytes per cell
    // Connected-component labelling of the solid mask, by kernel: run starts
    // (solid 1 -> label 4), links (solid 1), roots and classes (solid 1 ->
    // class 1); with an outlet the top marks (clear 1).  Labels other than
    // the run starts are not read again.
    const bool top_open = ctx->outlet && !(ctx->grid.periodic & 4);
    const double topo_bytes = 8.0 + (top_open ? 1.0 : 0.0);
    const double mask_bytes = ctx->ref ? 4.0 : 1.0;
    const Item classic[] = {
        {"spmv_dot", 20.0, 1, 0},             // p 4 + beta 12 -> q 4
        {"update_norm", 24.0, 1, 1},          // e, p, r, q 16 -> e, r 8
        {"fine_smooth_half", 12.0 + cb, 4, 2},  // r 4 + coef + z 4 -> z 4
        {"fine_restrict", 8.0 + cb + 0.25, 1, 3},
        {"fine_prolong", 8.25, 1, 4},
        {"dot_rz", 8.0, 1, 5},
        {"search", 12.0, 1, 6},
        {"refinement_residual", 24.0, 0, 7},  // x 4 + beta 12 + b 4 -> r 4 (survey K7)
        {"coefficients", 29.0, 0, 8},         // alpha 4 + solid 1 -> 16 + 8 (survey K0)
        {"topology", topo_bytes, 0, 9},
    };
    const Item pipelined[] = {
        // z 4 + p_old 4 + coef 16 + x 4 -> p 4 + x 4 + q 4
        {"search_spmv", 40.0, 1, 10},
        // r 4 + q 4 + coef -> r 4 + e 4 + coarse r (1/8 cell)
        {"presmooth_restrict", 16.0 + cb + vbc / 8.0, 1, 11},
        // e 4 + coarse e (1/8 cell) + r 4 + coef -> z 4
        {"prolong_postsmooth", 12.0 + cb + vbc / 8.0, 1, 12},
        // b 8 + x 8 (double-FP32 pairs) + coef 16 -> r 4 + e 4
        {"refinement_residual", 40.0, 0, 7},
        {"coefficients", 29.0, 0, 8},
        {"topology", topo_bytes, 0, 9},
        // fluid step (after a step has run): per axis launch, the three face
        // arrays 12 + fluid mask + the axis's output 4
        {"step_predict", 3.0 * (16.0 + mask_bytes), 0, 20},
        {"step_viscous", 3.0 * (16.0 + mask_bytes), 0, 21},
        // faces 12 + mask + potential 4 (+ liquid fraction 4) -> reductions
        {"step_fields", 20.0 + mask_bytes, 0, 22},
        // the coarse-grid correction of one V-cycle (every level below the
        // finest, W-cycle visits and bottom sub-cycle included) and one bottom
        // sub-cycle launch: latency-bound, no byte model
        {"coarse_levels", 0.0, 0, 13},
        {"bottom_subcycle", 0.0, 0, 14},
    };
    const Item* items = ctx->pipelined ? pipelined : classic;
    const int n_items = ctx->pipelined ? (int)(sizeof pipelined / sizeof pipelined[0])
                                       : (int)(sizeof classic / sizeof classic[0]);
    int k = 0;
    for (int ii = 0; ii < n_items; ii++) {
        const Item& it = items[ii];
        if (k >= max_out) break;
        if (!ctx->use_mg && (it.kind >= 2 && it.kind <= 4)) continue;
        if (it.kind >= 20 && it.kind <= 22 && !ctx->step_ran) continue;
        if (it.kind == 14 && ctx->mg.bottom_from <= 0) continue;
        launch_set_sigma(ctx->sc, 1.0f, s);  // clears the converged flag
        if (it.kind >= 10) launch_profile_reset(ctx->sc, s);
        // Timed as `reps` launches inside one CUDA graph, each after a small
        // reset kernel that clears the stop flags (a repeated launch of a
        // pass on unrelated inputs may meet a stop condition); a second graph
        // of the resets alone is timed and subtracted, so the time per launch
        // is the kernel's own duration plus the graph's launch spacing.
        const bool graphed = it.kind >= 7;
        if (graphed) {
            float ms_pair[2] = {0.f, 0.f};
            for (int pass = 0; pass < 2; pass++) {
                cudaGraph_t gr = nullptr;
                cudaGraphExec_t ge = nullptr;
                CK(cudaStreamSynchronize(s));
                cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
                if (e == cudaSuccess) {
                    for (int r = 0; r < reps; r++) {
                        launch_profile_reset(ctx->sc, s, true);
                        if (pass == 0) profile_launch(ctx, it.kind, r, F, s);
                    }
                    e = cudaStreamEndCapture(s, &gr);
                }
                if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, gr, 0);
                if (gr) cudaGraphDestroy(gr);
                if (e == cudaSuccess) e = cudaGraphLaunch(ge, s);  // warm-up
                if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_a, s);
                if (e == cudaSuccess) e = cudaGraphLaunch(ge, s);
                if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_b, s);
                if (e == cudaSuccess) e = cudaEventSynchronize(ctx->ev_b);
                if (e == cudaSuccess) e = cudaEventElapsedTime(&ms_pair[pass], ctx->ev_a, ctx->ev_b);
                if (ge) cudaGraphExecDestroy(ge);
                CK(e);
            }
            const float ms = std::max(ms_pair[0] - ms_pair[1], 0.0f);
            mhdproj_kernel_time& o = out[k++];
            memset(&o, 0, sizeof o);
            snprintf(o.name, sizeof o.name, "%s", it.name);
            o.ms = ms / reps;
            o.bytes = it.bytes_per_cell * n;
            o.per_iteration = it.per_it;
            continue;
        } else {
        CK(cudaEventRecord(ctx->ev_a, s));
        for (int r = 0; r < reps; r++) {
            profile_launch(ctx, it.kind, r, F, s);
            if (it.kind == 1 || it.kind == 5 || it.kind == 7) launch_set_sigma(ctx->sc, 1.0f, s);
            if (it.kind >= 10) launch_profile_reset(ctx->sc, s);
        }
        CK(cudaEventRecord(ctx->ev_b, s));
        }
        CK(cudaGetLastError());
        int rc = wait_stream(ctx);
        if (rc) return rc;
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, ctx->ev_a, ctx->ev_b));
        mhdproj_kernel_time& o = out[k++];
        memset(&o, 0, sizeof o);
        snprintf(o.name, sizeof o.name, "%s", it.name);
        o.ms = ms / reps;
        o.bytes = it.bytes_per_cell * n;
        o.per_iteration = it.per_it;
    }
    *count = k;
    ctx->have_solution = false;
    return 0;
}

extern "C" int mhdproj_kernel_launches(mhdproj_ctx* ctx, uint64_t* count) {
    if (!ctx || !count) return MHDPROJ_ERR_INVALID;
    *count = ctx->launches;
    return 0;
}

// ------------------------------------------------------------ utilities
extern "C" int mhdproj_hierarchy(const uint32_t dims[4], uint32_t* levels, uint64_t* coarse_cells) {
    return host_hierarchy(dims, levels, coarse_cells) ? MHDPROJ_ERR_INVALID : 0;
}
extern "C" uint32_t mhdproj_anchors(uint32_t* mask, const uint32_t dims[3], uint32_t periodic) {
    return host_anchors(mask, dims, periodic);
}
