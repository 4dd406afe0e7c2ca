// gb300_kernels.cu -- fine-level kernels of the GB300 projection.
//
// Layout in HBM (x-fastest, cell i = x + nx*(y + ny*z)):
//   coef  float4[n]  (beta_x, beta_y, beta_z of the low faces, reaction)
//   cls   uint8[n]   0 solid, 1 active, 2 pinned gauge cell
//   b (hi, lo), phi (hi, lo) float[n] pairs; r, z, p, q, e float[n]
//   faces u[(nx+1) ny nz], v[nx (ny+1) nz], w[nx ny (nz+1)]
// Every kernel walks 32x8 (x, y) tiles over a run of z, so warps read 128-byte
// rows and neighbouring z-planes are reused from L2.  Reductions take
// error-free FP32 products and compensated sums per thread, then FP64 warp
// shuffles, one partial per block, and a deterministic fixed-order sum in the
// last block, which also updates the CG scalars.  Quantities that need more
// than FP32 (right-hand side, accumulated potential, refinement residual) are
// double-FP32 pairs (see common.cuh).
#include "kernels.h"

namespace mhdproj {

#define TILE_BEGIN(G)                                      \
    const int x = blockIdx.x * TX + threadIdx.x;           \
    const int y = blockIdx.y * TY + threadIdx.y;           \
    const bool in_xy = x < (G).nx && y < (G).ny;           \
    const int z0 = blockIdx.z * (G).zper;                  \
    const int z1 = min((G).nz, z0 + (G).zper);             \
    for (int z = z0; z < z1; z++)
// A thread's (x, y) column and z run, for kernels that walk the run two
// planes at a time: both planes' loads are issued before either plane's
// arithmetic (the one-pass set-up kernels are bound by memory latency).
#define TILE_COLUMN(G)                                     \
    const int x = blockIdx.x * TX + threadIdx.x;           \
    const int y = blockIdx.y * TY + threadIdx.y;           \
    const bool in_xy = x < (G).nx && y < (G).ny;           \
    const int z0 = blockIdx.z * (G).zper;                  \
    const int z1 = min((G).nz, z0 + (G).zper)
// Runs load(z) -> In and finish(z, In) over the column's planes in pairs.
template <class Load, class Finish>
__device__ __forceinline__ void walk_pairs(int z0, int z1, Load load, Finish finish) {
    int z = z0;
    for (; z + 1 < z1; z += 2) {
        const auto a = load(z);
        const auto b = load(z + 1);
        finish(z, a);
        finish(z + 1, b);
    }
    if (z < z1) finish(z, load(z));
}

__device__ __forceinline__ int cell_index(const Grid3& g, int x, int y, int z) { return x + g.nx * (y + g.ny * z); }

struct Nbr {
    int xm, xp, ym, yp, zm, zp;  // neighbour cell index or -1
};
__device__ __forceinline__ Nbr neighbours(const Grid3& g, int x, int y, int z) {
    Nbr n;
    const int sx = 1, sy = g.nx, sz = g.nx * g.ny;
    const int i = x + sy * y + sz * z;
    int c;
    c = wrap_or_neg(x - 1, g.nx, g.periodic & 1); n.xm = c < 0 ? -1 : i + (c - x) * sx;
    c = wrap_or_neg(x + 1, g.nx, g.periodic & 1); n.xp = c < 0 ? -1 : i + (c - x) * sx;
    c = wrap_or_neg(y - 1, g.ny, g.periodic & 2); n.ym = c < 0 ? -1 : i + (c - y) * sy;
    c = wrap_or_neg(y + 1, g.ny, g.periodic & 2); n.yp = c < 0 ? -1 : i + (c - y) * sy;
    c = wrap_or_neg(z - 1, g.nz, g.periodic & 4); n.zm = c < 0 ? -1 : i + (c - z) * sz;
    c = wrap_or_neg(z + 1, g.nz, g.periodic & 4); n.zp = c < 0 ? -1 : i + (c - z) * sz;
    return n;
}

// ------------------------------------------------------------- scalars
__global__ void k_init_scalars(Scalars* sc, double tol2, double abs_floor, double inner_floor2, int max_total) {
    sc->tol2 = tol2;
    sc->max_total = max_total;
    sc->inv_sigma_z = 1.0f;
    sc->first = 1;
    sc->pidx = 0;
    sc->abs_floor = abs_floor;
    sc->inner_floor2 = inner_floor2;
    sc->total_iterations = 0;
    sc->iterations = 0;
    sc->converged = 0;
    sc->outer_done = 0;
    sc->nonfinite = 0;
    sc->breakdown = 0;
    sc->sigma = 1.0f;
    sc->inv_sigma = 1.0f;
    sc->alpha = sc->beta = 0.0;
    sc->alpha_f = sc->beta_f = 0.0f;
}
__global__ void k_set_sigma(Scalars* sc, float sigma) {
    sc->sigma = sigma;
    sc->inv_sigma = 1.0f / sigma;
    sc->converged = 0;
}

// ------------------------------------------------------- coefficients
__global__ void __launch_bounds__(TILE_THREADS) k_coefficients(Grid3 g, int outlet, const float* __restrict__ alpha,
                                                               const uint8_t* __restrict__ cls, Mobility mob,
                                                               float4* __restrict__ coef,
                                                               void* __restrict__ lo, int lo_kind,
                                                               float* __restrict__ gtop) {
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        const Nbr nb = neighbours(g, x, y, z);
        float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
        // every load first (guarded by the coordinates only), so the cell's
        // loads are in flight together
        const uint8_t ci = cls[i];
        const float ai = alpha[i];
        const int order[6] = {nb.xm, nb.xp, nb.ym, nb.yp, nb.zm, nb.zp};
        uint8_t cn[6];
        float an[6];
#pragma unroll
        for (int k = 0; k < 6; k++) {
            cn[k] = order[k] >= 0 ? cls[order[k]] : (uint8_t)0;
            an[k] = order[k] >= 0 ? alpha[order[k]] : 0.0f;
        }
        if (ci == 1) {
            if (cn[0] == 1) c.x = mobility_of(mob, an[0], ai, order[0], i);
            if (cn[2] == 1) c.y = mobility_of(mob, an[2], ai, order[2], i);
            if (cn[4] == 1) c.z = mobility_of(mob, an[4], ai, order[4], i);
            float r = 0.0f;
#pragma unroll
            for (int k = 0; k < 6; k++)
                if (cn[k] == 2) r = __fadd_rn(r, mobility_of(mob, ai, an[k], i, order[k]));
            if (outlet && z == g.nz - 1) {
                const float gt = outlet_mobility(mob, ai, i);
                r = __fadd_rn(r, gt);
                gtop[x + g.nx * y] = gt;
            }
            c.w = r;
        } else if (outlet && z == g.nz - 1) {
            gtop[x + g.nx * y] = 0.0f;
        }
        coef[i] = c;
        if (lo_kind == 1) reinterpret_cast<uint2*>(lo)[i] = pack_coef_h(c);
        else if (lo_kind == 2) reinterpret_cast<uint2*>(lo)[i] = pack_coef_b(c);
    }
}

// ------------------------------------------------------------------ rhs
// b = -h * sum over open faces of (u_high - u_low) as a double-FP32 pair;
// ||b||^2.
// start_pass: the solve starts from x = 0, so this kernel also sets up its
// first pass: r = b (rounded to FP32), x = 0 and the pass scalars of
// k_residual with ||b - A 0||^2 = ||b||^2.
__global__ void __launch_bounds__(TILE_THREADS) k_rhs(Grid3 g, int outlet, float h, const uint8_t* __restrict__ cls,
                                                      const float* __restrict__ u, const float* __restrict__ v,
                                                      const float* __restrict__ w, float* __restrict__ b_hi,
                                                      float* __restrict__ b_lo, float* __restrict__ r,
                                                      float* __restrict__ xs, int start_pass, Scalars* sc,
                                                      double* partials, int nblocks, long long n_active) {
    __shared__ double sh[8 * 1];
    Acc acc;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    TILE_COLUMN(g);
    struct In {
        float ulo, uhi, vlo, vhi, wlo, whi;
        uint8_t ci, cxm, cxp, cym, cyp, czm, czp;
        bool zp_in;  // the cell above exists (not the top of a closed z axis)
    };
    // every load of a cell first (face indices are always valid)
    auto load = [&](int z) {
        In L;
        const int i = cell_index(g, x, y, z);
        const Nbr nb = neighbours(g, x, y, z);
        L.ci = cls[i];
        L.cxm = nb.xm >= 0 ? cls[nb.xm] : 0;
        L.cxp = nb.xp >= 0 ? cls[nb.xp] : 0;
        L.cym = nb.ym >= 0 ? cls[nb.ym] : 0;
        L.cyp = nb.yp >= 0 ? cls[nb.yp] : 0;
        L.czm = nb.zm >= 0 ? cls[nb.zm] : 0;
        L.czp = nb.zp >= 0 ? cls[nb.zp] : 0;
        L.zp_in = nb.zp >= 0;
        const int hx = (x + 1 == nx && (g.periodic & 1)) ? 0 : x + 1;
        const int hy = (y + 1 == ny && (g.periodic & 2)) ? 0 : y + 1;
        const int hz = (z + 1 == nz && (g.periodic & 4)) ? 0 : z + 1;
        L.ulo = u[x + (nx + 1) * (y + ny * z)];
        L.uhi = u[hx + (nx + 1) * (y + ny * z)];
        L.vlo = v[x + nx * (y + (ny + 1) * z)];
        L.vhi = v[x + nx * (hy + (ny + 1) * z)];
        L.wlo = w[x + nx * (y + ny * z)];
        L.whi = w[x + nx * (y + ny * hz)];
        return L;
    };
    auto finish = [&](int z, const In& L) {
        const int i = cell_index(g, x, y, z);
        df bi = {0.0f, 0.0f};
        if (L.ci == 1) {
            df sum = {0.0f, 0.0f};
            sum = df_add(sum, two_sum(L.cxp != 0 ? L.uhi : 0.0f, -(L.cxm != 0 ? L.ulo : 0.0f)));
            sum = df_add(sum, two_sum(L.cyp != 0 ? L.vhi : 0.0f, -(L.cym != 0 ? L.vlo : 0.0f)));
            const bool hopen = (L.zp_in && L.czp != 0) || (!L.zp_in && outlet && z + 1 == nz);
            sum = df_add(sum, two_sum(hopen ? L.whi : 0.0f, -(L.czm != 0 ? L.wlo : 0.0f)));
            bi = df_mul_f(sum, -h);
        }
        b_hi[i] = bi.hi;
        b_lo[i] = bi.lo;
        acc.add_prod(bi.hi, bi.hi);
        if (start_pass) {
            r[i] = df_to_f(bi);
            xs[i] = 0.0f;
        }
    };
    if (in_xy) walk_pairs(z0, z1, load, finish);
    double v1[1] = {acc.total()};
    block_sum<1>(v1, sh);
    if (store_partials_is_last<1>(v1, partials, nblocks, &sc->ticket[0])) {
        double tot[1];
        finish_partials<1>(tot, partials, nblocks, sh, &sc->ticket[0]);
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            const double bb = tot[0];
            sc->bb = bb;
            if (!isfinite(bb)) sc->nonfinite = 1;
            if (start_pass) {
                sc->rr_true = bb;
                sc->rr = bb;
                sc->iterations = 0;
                const double goal = sc->tol2 * bb + sc->abs_floor;
                const bool done = !(bb > goal) || bb == 0.0;
                sc->outer_done = done ? 1 : 0;
                sc->converged = (done || !isfinite(bb)) ? 1 : 0;
                sc->rr_target = fmax(sc->inner_floor2 * bb, 0.25 * goal);
                set_sigma_from(sc, bb, n_active);
                sc->first = 1;
                sc->alpha = sc->beta = 0.0;
                sc->alpha_f = sc->beta_f = 0.0f;
            }
        }
    }
}

// y = A x with the FP32 coefficients, in FP64 (T = double) or FP32.
template <class T>
__device__ __forceinline__ T apply_cell(const Grid3& g, const float4* __restrict__ coef, const T* __restrict__ xv,
                                        int i, const Nbr& nb) {
    const float4 c = coef[i];
    const T xi = xv[i];
    T acc = (T)c.w * xi;
    if (c.x != 0.f) acc += (T)c.x * (xi - xv[nb.xm]);
    if (c.y != 0.f) acc += (T)c.y * (xi - xv[nb.ym]);
    if (c.z != 0.f) acc += (T)c.z * (xi - xv[nb.zm]);
    if (nb.xp >= 0) { const float bh = coef[nb.xp].x; if (bh != 0.f) acc += (T)bh * (xi - xv[nb.xp]); }
    if (nb.yp >= 0) { const float bh = coef[nb.yp].y; if (bh != 0.f) acc += (T)bh * (xi - xv[nb.yp]); }
    if (nb.zp >= 0) { const float bh = coef[nb.zp].z; if (bh != 0.f) acc += (T)bh * (xi - xv[nb.zp]); }
    return acc;
}

// ------------------------------------------------- refinement residual
// x_i - x_j in double-FP32, left unnormalised: TwoSum of the high parts, the
// low parts' difference added to its error.
__device__ __forceinline__ df df_diff_lazy(df a, df b) {
    const df s = two_sum(a.hi, -b.hi);
    return {s.hi, __fadd_rn(s.lo, __fsub_rn(a.lo, b.lo))};
}
// acc += beta * d: the high product exact (FMA TwoProduct), added by TwoSum;
// the low terms gathered in acc.lo (renormalised once at the end).
__device__ __forceinline__ void df_acc_prod(df& acc, df d, float beta) {
    const float p = __fmul_rn(d.hi, beta);
    const float pl = __fmaf_rn(d.lo, beta, __fmaf_rn(d.hi, beta, -p));
    const df s = two_sum(acc.hi, p);
    acc = {s.hi, __fadd_rn(acc.lo, __fadd_rn(s.lo, pl))};
}

// r = b - A x in double-FP32 (x a double-FP32 pair), stored FP32 for the
// inner solve; e = 0.  Every load of a cell is issued before its arithmetic
// (an absent neighbour sits behind a zero mobility and reads as x_i), and
// the seven terms are gathered with lazy double-FP32 sums (about 2^-44
// relative to the largest term).
__global__ void __launch_bounds__(TILE_THREADS) k_residual(Grid3 g, const float4* __restrict__ coef,
                                                           const float* __restrict__ b_hi,
                                                           const float* __restrict__ b_lo,
                                                           const float* __restrict__ x_hi,
                                                           const float* __restrict__ x_lo, float* __restrict__ r,
                                                           float* __restrict__ e, Scalars* sc, double* partials,
                                                           int nblocks, long long n_active) {
    __shared__ double sh[8 * 1];
    Acc acc;
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        const Nbr nb = neighbours(g, x, y, z);
        const float4 c = coef[i];
        const float bxp = nb.xp >= 0 ? coef[nb.xp].x : 0.f;
        const float byp = nb.yp >= 0 ? coef[nb.yp].y : 0.f;
        const float bzp = nb.zp >= 0 ? coef[nb.zp].z : 0.f;
        const df xi = {x_hi[i], x_lo[i]};
        auto ld = [&](int j) { return j >= 0 ? df{x_hi[j], x_lo[j]} : xi; };
        const df xxm = ld(nb.xm), xxp = ld(nb.xp), xym = ld(nb.ym), xyp = ld(nb.yp), xzm = ld(nb.zm), xzp = ld(nb.zp);
        const df bi = {b_hi[i], b_lo[i]};
        df ax;
        ax.hi = __fmul_rn(xi.hi, c.w);
        ax.lo = __fmaf_rn(xi.lo, c.w, __fmaf_rn(xi.hi, c.w, -ax.hi));
        df_acc_prod(ax, df_diff_lazy(xi, xxm), c.x);
        df_acc_prod(ax, df_diff_lazy(xi, xym), c.y);
        df_acc_prod(ax, df_diff_lazy(xi, xzm), c.z);
        df_acc_prod(ax, df_diff_lazy(xi, xxp), bxp);
        df_acc_prod(ax, df_diff_lazy(xi, xyp), byp);
        df_acc_prod(ax, df_diff_lazy(xi, xzp), bzp);
        const df res = df_sub(bi, fast_two_sum(ax.hi, ax.lo));
        const float ri = df_to_f(res);
        r[i] = ri;
        e[i] = 0.0f;
        acc.add_prod(ri, ri);
    }
    double v1[1] = {acc.total()};
    block_sum<1>(v1, sh);
    if (store_partials_is_last<1>(v1, partials, nblocks, &sc->ticket[1])) {
        double tot[1];
        finish_partials<1>(tot, partials, nblocks, sh, &sc->ticket[1]);
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            const double rr = tot[0];
            sc->rr_true = rr;
            sc->rr = rr;
            sc->iterations = 0;
            const double goal = sc->tol2 * sc->bb + sc->abs_floor;
            const bool done = !(rr > goal) || sc->bb == 0.0;
            sc->outer_done = done ? 1 : 0;
            if (!isfinite(rr)) sc->nonfinite = 1;
            sc->converged = (done || !isfinite(rr)) ? 1 : 0;
            sc->rr_target = fmax(sc->inner_floor2 * rr, 0.25 * goal);
            set_sigma_from(sc, rr, n_active);
            // a new CG pass: the first search direction is z itself
            sc->first = 1;
            sc->alpha = sc->beta = 0.0;
            sc->alpha_f = sc->beta_f = 0.0f;
        }
    }
}

// --------------------------------------------------------- CG kernels
// q = A p and p.q.  Each thread marches its column along z keeping p at
// z-1, z, z+1 and the coefficient records at z, z+1 in registers and loading
// plane z+2 one step ahead; in-plane neighbours come from L1.
__global__ void __launch_bounds__(TILE_THREADS) k_spmv_pq(Grid3 g, const float4* __restrict__ coef,
                                                          const float* __restrict__ p, float* __restrict__ q,
                                                          Scalars* sc, double* partials, int nblocks) {
    if (sc->converged) return;
    __shared__ double sh[8 * 1];
    Acc acc;
    const int x = blockIdx.x * TX + threadIdx.x, y = blockIdx.y * TY + threadIdx.y;
    const int z0 = blockIdx.z * g.zper, z1 = min(g.nz, z0 + g.zper);
    if (x < g.nx && y < g.ny) {
        const Column C(g, x, y);
        const float* coefs = reinterpret_cast<const float*>(coef);
        const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
        float pm = p[C.zat(z0 - 1)], pc = p[C.at(z0)], pn = p[C.zat(z0 + 1)];
        float4 cc = coef[C.at(z0)];
        float4 cn = C.zexists(z0 + 1) ? coef[C.zat(z0 + 1)] : zero4;
        for (int z = z0; z < z1; z++) {
            const int i = C.at(z);
            float pnn = 0.f;
            float4 cnn = zero4;
            if (z + 1 < z1) {
                pnn = p[C.zat(z + 2)];
                if (C.zexists(z + 2)) cnn = coef[C.zat(z + 2)];
            }
            const float pxm = p[i + C.dxm], pxp = p[i + C.dxp], pym = p[i + C.dym], pyp = p[i + C.dyp];
            const float bxh = C.hxp ? coefs[4 * (i + C.dxp)] : 0.f;
            const float byh = C.hyp ? coefs[4 * (i + C.dyp) + 1] : 0.f;
            float qv = cc.w * pc;
            qv = fmaf(cc.x, pc - pxm, qv);
            qv = fmaf(bxh, pc - pxp, qv);
            qv = fmaf(cc.y, pc - pym, qv);
            qv = fmaf(byh, pc - pyp, qv);
            qv = fmaf(cc.z, pc - pm, qv);
            qv = fmaf(cn.z, pc - pn, qv);
            q[i] = qv;
            acc.add_prod(pc, qv);
            pm = pc;
            pc = pn;
            pn = pnn;
            cc = cn;
            cn = cnn;
        }
    }
    double v1[1] = {acc.total()};
    block_sum<1>(v1, sh);
    if (store_partials_is_last<1>(v1, partials, nblocks, &sc->ticket[2])) {
        double tot[1];
        finish_partials<1>(tot, partials, nblocks, sh, &sc->ticket[2]);
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            const double pq = tot[0];
            sc->pq = pq;
            if (!(pq > 0.0) || !isfinite(pq)) {
                sc->breakdown = 1;
                if (!isfinite(pq)) sc->nonfinite = 1;
                sc->converged = 1;
                sc->alpha = 0.0;
                sc->alpha_f = 0.0f;
            } else {
                sc->alpha = sc->rz / pq;
                sc->alpha_f = (float)sc->alpha;
            }
        }
    }
}

// Streaming kernels walk the column four planes at a time with all loads
// issued before any store, so each thread keeps several requests in flight.
#define STREAM_BEGIN(G)                                                             \
    const int x = blockIdx.x * TX + threadIdx.x, y = blockIdx.y * TY + threadIdx.y; \
    const int z0 = blockIdx.z * (G).zper, z1 = min((G).nz, z0 + (G).zper);          \
    const int sxy = (G).nx * (G).ny;                                                \
    const bool inside = x < (G).nx && y < (G).ny;                                   \
    const int base = x + (G).nx * y;

// The vector updates and dot products are pure streams: flat grid-stride
// loops over float4 chunks give long contiguous bursts (the column walk of the
// stencil kernels would scatter 128-byte requests over many DRAM pages).
constexpr int FLAT_BLOCKS = 152 * 8;

__global__ void __launch_bounds__(256) k_update(long long n, float* __restrict__ e, float* __restrict__ r,
                                                const float* __restrict__ p, const float* __restrict__ q, Scalars* sc,
                                                double* partials, int nblocks, long long n_active) {
    if (sc->converged) return;
    __shared__ double sh[8 * 1];
    Acc acc;
    const float a = sc->alpha_f;
    const long long n4 = n >> 2;
    const long long stride = (long long)gridDim.x * blockDim.x;
    float4* e4 = reinterpret_cast<float4*>(e);
    float4* r4 = reinterpret_cast<float4*>(r);
    const float4* p4 = reinterpret_cast<const float4*>(p);
    const float4* q4 = reinterpret_cast<const float4*>(q);
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n4; k += stride) {
        const float4 ev = e4[k], rv = r4[k], pv = p4[k], qv = q4[k];
        const float4 en = make_float4(fmaf(a, pv.x, ev.x), fmaf(a, pv.y, ev.y), fmaf(a, pv.z, ev.z), fmaf(a, pv.w, ev.w));
        const float4 rn = make_float4(fmaf(-a, qv.x, rv.x), fmaf(-a, qv.y, rv.y), fmaf(-a, qv.z, rv.z),
                                      fmaf(-a, qv.w, rv.w));
        e4[k] = en;
        r4[k] = rn;
        acc.add_prod(rn.x, rn.x);
        acc.add_prod(rn.y, rn.y);
        acc.add_prod(rn.z, rn.z);
        acc.add_prod(rn.w, rn.w);
    }
    if (blockIdx.x == 0 && threadIdx.x < (n & 3)) {
        const long long i = (n4 << 2) + threadIdx.x;
        e[i] = fmaf(a, p[i], e[i]);
        const float ri = fmaf(-a, q[i], r[i]);
        r[i] = ri;
        acc.add_prod(ri, ri);
    }
    double v1[1] = {acc.total()};
    block_sum<1>(v1, sh);
    if (store_partials_is_last<1>(v1, partials, nblocks, &sc->ticket[3])) {
        double tot[1];
        finish_partials<1>(tot, partials, nblocks, sh, &sc->ticket[3]);
        if (threadIdx.x == 0) {
            const double rr = tot[0];
            sc->rr = rr;
            sc->iterations += 1;
            sc->total_iterations += 1;
            if (!isfinite(rr)) {
                sc->nonfinite = 1;
                sc->converged = 1;
            } else if (rr <= sc->rr_target) {
                sc->converged = 1;
            }
            set_sigma_from(sc, rr, n_active);
        }
    }
}

// rz = r . z / sigma; init: p = z / sigma.
__global__ void __launch_bounds__(256) k_dot_rz(long long n, const float* __restrict__ r, const float* __restrict__ zv,
                                                float* __restrict__ p, int init, Scalars* sc, double* partials,
                                                int nblocks) {
    if (sc->converged) return;
    __shared__ double sh[8 * 1];
    Acc acc;
    const float is = sc->inv_sigma;
    const long long n4 = n >> 2;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const float4* r4 = reinterpret_cast<const float4*>(r);
    const float4* z4 = reinterpret_cast<const float4*>(zv);
    float4* p4 = reinterpret_cast<float4*>(p);
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n4; k += stride) {
        const float4 rv = r4[k], zz = z4[k];
        const float4 zs = make_float4(zz.x * is, zz.y * is, zz.z * is, zz.w * is);
        if (init) p4[k] = zs;
        acc.add_prod(rv.x, zs.x);
        acc.add_prod(rv.y, zs.y);
        acc.add_prod(rv.z, zs.z);
        acc.add_prod(rv.w, zs.w);
    }
    if (blockIdx.x == 0 && threadIdx.x < (n & 3)) {
        const long long i = (n4 << 2) + threadIdx.x;
        const float zi = zv[i] * is;
        if (init) p[i] = zi;
        acc.add_prod(r[i], zi);
    }
    double v1[1] = {acc.total()};
    block_sum<1>(v1, sh);
    if (store_partials_is_last<1>(v1, partials, nblocks, &sc->ticket[4])) {
        double tot[1];
        finish_partials<1>(tot, partials, nblocks, sh, &sc->ticket[4]);
        if (threadIdx.x == 0) {
            const double rz = tot[0];
            if (!isfinite(rz)) {
                sc->nonfinite = 1;
                sc->converged = 1;
            } else if (!(rz > 0.0)) {
                sc->breakdown = 1;
                sc->converged = 1;
            } else if (init) {
                sc->rz = rz;
            } else {
                sc->beta = rz / sc->rz;
                sc->beta_f = (float)sc->beta;
                sc->rz = rz;
            }
        }
    }
}

__global__ void __launch_bounds__(256) k_search(long long n, const float* __restrict__ zv, float* __restrict__ p,
                                                const Scalars* sc) {
    if (sc->converged) return;
    const float is = sc->inv_sigma, bt = sc->beta_f;
    const long long n4 = n >> 2;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const float4* z4 = reinterpret_cast<const float4*>(zv);
    float4* p4 = reinterpret_cast<float4*>(p);
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n4; k += stride) {
        const float4 zz = z4[k], pv = p4[k];
        p4[k] = make_float4(fmaf(bt, pv.x, zz.x * is), fmaf(bt, pv.y, zz.y * is), fmaf(bt, pv.z, zz.z * is),
                            fmaf(bt, pv.w, zz.w * is));
    }
    if (blockIdx.x == 0 && threadIdx.x < (n & 3)) {
        const long long i = (n4 << 2) + threadIdx.x;
        p[i] = fmaf(bt, p[i], zv[i] * is);
    }
}

__global__ void __launch_bounds__(TILE_THREADS) k_accumulate(Grid3 g, float* __restrict__ x_hi,
                                                             float* __restrict__ x_lo, const float* __restrict__ e) {
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        const df v = df_add_f(df{x_hi[i], x_lo[i]}, e[i]);
        x_hi[i] = v.hi;
        x_lo[i] = v.lo;
    }
}
// End of a pipelined CG pass: the last step's x += alpha p is still pending
// (the search kernel applies it one step late), so phi += x + alpha p.
__global__ void __launch_bounds__(TILE_THREADS) k_accumulate_pipelined(Grid3 g, float* __restrict__ x_hi,
                                                                       float* __restrict__ x_lo,
                                                                       const float* __restrict__ e,
                                                                       const float* __restrict__ p0,
                                                                       const float* __restrict__ p1,
                                                                       const Scalars* sc) {
    const float a = sc->alpha_f;
    const float* p = sc->pidx ? p1 : p0;
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        const float ev = a != 0.0f ? fmaf(a, p[i], e[i]) : e[i];
        const df v = df_add_f(df{x_hi[i], x_lo[i]}, ev);
        x_hi[i] = v.hi;
        x_lo[i] = v.lo;
    }
}
__global__ void k_to_double(const float* __restrict__ hi, const float* __restrict__ lo, double* __restrict__ out,
                            long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = (double)hi[i] + (double)lo[i];
}

__global__ void __launch_bounds__(TILE_THREADS) k_apply(Grid3 g, const float4* __restrict__ coef,
                                                        const float* __restrict__ xv, float* __restrict__ yv) {
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        yv[i] = apply_cell<float>(g, coef, xv, i, neighbours(g, x, y, z));
    }
}
__global__ void __launch_bounds__(TILE_THREADS) k_scale(Grid3 g, const float* __restrict__ in, float* __restrict__ out,
                                                        float scale, const Scalars* sc) {
    const float s = sc ? sc->inv_sigma : scale;
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        out[i] = in[i] * s;
    }
}

// ---------------------------------------------------- gradient subtraction
// u = u* - beta (phi_R - phi_L) / h on open faces, the outlet face uses its
// conductance against p = 0 on the face, closed faces are 0.  Potential
// differences are taken in double-FP32 before rounding.  Each thread owns the
// low faces of its cell; the thread at index 0 of a periodic axis also writes
// the duplicate last face, the thread at the high end of a closed axis writes
// that wall face.
__device__ __forceinline__ float grad_term(float bt, df pi, df pj, float inv_h) {
    return __fmul_rn(__fmul_rn(bt, df_to_f(df_sub(pi, pj))), inv_h);
}
__global__ void __launch_bounds__(TILE_THREADS) k_correct(Grid3 g, int outlet, float h, Mobility mob,
                                                          float p_scale, const uint8_t* __restrict__ cls,
                                                          const float* __restrict__ alpha,
                                                          const float* __restrict__ gtop,
                                                          const float* __restrict__ ph, const float* __restrict__ pl,
                                                          const float* __restrict__ us, const float* __restrict__ vs,
                                                          const float* __restrict__ ws, float* __restrict__ uo,
                                                          float* __restrict__ vo, float* __restrict__ wo,
                                                          float* __restrict__ po) {
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const float inv_h = 1.0f / h;
    TILE_COLUMN(g);
    struct In {
        df pi, pxm, pym, pzm;
        float ai, axm, aym, azm, uin, vin, win;
        int xm, ym, zm;  // low neighbours or -1
        uint8_t ci, cxm, cym, czm;
    };
    // every load of a cell first (guarded by the coordinates only)
    auto load = [&](int z) {
        In L;
        const int i = cell_index(g, x, y, z);
        const Nbr nb = neighbours(g, x, y, z);
        L.xm = nb.xm;
        L.ym = nb.ym;
        L.zm = nb.zm;
        L.ci = cls[i];
        L.pi = {ph[i], pl[i]};
        L.ai = alpha[i];
        L.cxm = nb.xm >= 0 ? cls[nb.xm] : 0;
        L.cym = nb.ym >= 0 ? cls[nb.ym] : 0;
        L.czm = nb.zm >= 0 ? cls[nb.zm] : 0;
        L.axm = nb.xm >= 0 ? alpha[nb.xm] : 0.f;
        L.aym = nb.ym >= 0 ? alpha[nb.ym] : 0.f;
        L.azm = nb.zm >= 0 ? alpha[nb.zm] : 0.f;
        L.pxm = nb.xm >= 0 ? df{ph[nb.xm], pl[nb.xm]} : L.pi;
        L.pym = nb.ym >= 0 ? df{ph[nb.ym], pl[nb.ym]} : L.pi;
        L.pzm = nb.zm >= 0 ? df{ph[nb.zm], pl[nb.zm]} : L.pi;
        L.uin = us[x + (nx + 1) * (y + ny * z)];
        L.vin = vs[x + nx * (y + (ny + 1) * z)];
        L.win = ws[x + nx * (y + ny * z)];
        return L;
    };
    auto finish = [&](int z, const In& L) {
        const int i = cell_index(g, x, y, z);
        {
            const int f = x + (nx + 1) * (y + ny * z);
            float out = 0.0f;
            if (L.xm >= 0 && L.ci != 0 && L.cxm != 0)
                out = L.uin - grad_term(mobility_of(mob, L.axm, L.ai, L.xm, i), L.pi, L.pxm, inv_h);
            uo[f] = out;
            if (x == 0 && (g.periodic & 1)) uo[nx + (nx + 1) * (y + ny * z)] = out;
            if (x == nx - 1 && !(g.periodic & 1)) uo[nx + (nx + 1) * (y + ny * z)] = 0.0f;
        }
        {
            const int f = x + nx * (y + (ny + 1) * z);
            float out = 0.0f;
            if (L.ym >= 0 && L.ci != 0 && L.cym != 0)
                out = L.vin - grad_term(mobility_of(mob, L.aym, L.ai, L.ym, i), L.pi, L.pym, inv_h);
            vo[f] = out;
            if (y == 0 && (g.periodic & 2)) vo[x + nx * (ny + (ny + 1) * z)] = out;
            if (y == ny - 1 && !(g.periodic & 2)) vo[x + nx * (ny + (ny + 1) * z)] = 0.0f;
        }
        {
            const int f = x + nx * (y + ny * z);
            float out = 0.0f;
            if (L.zm >= 0 && L.ci != 0 && L.czm != 0)
                out = L.win - grad_term(mobility_of(mob, L.azm, L.ai, L.zm, i), L.pi, L.pzm, inv_h);
            wo[f] = out;
            const int ft = x + nx * (y + ny * nz);
            if (z == 0 && (g.periodic & 4)) wo[ft] = out;
            if (z == nz - 1 && !(g.periodic & 4)) {
                float top = 0.0f;
                if (outlet && L.ci != 0) top = ws[ft] + __fmul_rn(__fmul_rn(gtop[x + nx * y], df_to_f(L.pi)), inv_h);
                wo[ft] = top;
            }
        }
        if (po) po[i] = L.ci != 0 ? __fmul_rn(p_scale, df_to_f(L.pi)) : 0.0f;
    };
    if (in_xy) walk_pairs(z0, z1, load, finish);
}

// max |div u| and sum div^2 over active cells of a face field.
__global__ void __launch_bounds__(TILE_THREADS) k_divergence(Grid3 g, float h, const uint8_t* __restrict__ cls,
                                                             const float* __restrict__ u, const float* __restrict__ v,
                                                             const float* __restrict__ w, Scalars* sc,
                                                             double* partials, int nblocks) {
    __shared__ double sh[8 * 2];
    __shared__ double shm[8];
    float mx = 0.0f;
    Acc acc;
    const int nx = g.nx, ny = g.ny;
    const float inv_h = 1.0f / h;
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        if (cls[i] != 1) continue;
        df d = two_sum(u[x + 1 + (nx + 1) * (y + ny * z)], -u[x + (nx + 1) * (y + ny * z)]);
        d = df_add(d, two_sum(v[x + nx * (y + 1 + (ny + 1) * z)], -v[x + nx * (y + (ny + 1) * z)]));
        d = df_add(d, two_sum(w[x + nx * (y + ny * (z + 1))], -w[x + nx * (y + ny * z)]));
        const float dv = df_to_f(d) * inv_h;
        mx = fmaxf(mx, fabsf(dv));
        acc.add_prod(dv, dv);
    }
    const int t = threadIdx.x + blockDim.x * threadIdx.y;
    double m = warp_max((double)mx);
    if ((t & 31) == 0) shm[t >> 5] = m;
    double v2[2] = {0.0, acc.total()};
    {
        double s1[1] = {v2[1]};
        block_sum<1>(s1, sh);  // contains the barrier that publishes shm
        v2[1] = s1[0];
    }
    if (t == 0) {
        double mm = 0.0;
        for (int k = 0; k < 8; k++) mm = fmax(mm, shm[k]);
        v2[0] = mm;
    }
    if (store_partials_is_last<2>(v2, partials, nblocks, &sc->ticket[5])) {
        __threadfence();
        double mb = 0.0, sb = 0.0;
        for (int b = t; b < nblocks; b += TILE_THREADS) {
            mb = fmax(mb, ((volatile double*)partials)[b]);
            sb += ((volatile double*)partials)[nblocks + b];
        }
        mb = warp_max(mb);
        __syncthreads();
        if ((t & 31) == 0) shm[t >> 5] = mb;
        double s1[1] = {sb};
        block_sum<1>(s1, sh);
        if (t == 0) {
            double mm = 0.0;
            for (int k = 0; k < 8; k++) mm = fmax(mm, shm[k]);
            sc->divmax = mm;
            sc->div2 = s1[0];
            sc->ticket[5] = 0u;
        }
    }
}

// ----------------------------------------------------------- adjoint
// g_phi = d u / d phi ^T g_u + rho_l/dt g_p on active cells (the transposed
// gradient), a double-FP32 right-hand side; ||b||^2.  Gradients of a periodic
// duplicate face are folded into the canonical face.
__global__ void __launch_bounds__(TILE_THREADS) k_adj_rhs(Grid3 g, int outlet, float h, Mobility mob,
                                                          float p_scale, const uint8_t* __restrict__ cls,
                                                          const float* __restrict__ alpha,
                                                          const float* __restrict__ gtop,
                                                          const float* __restrict__ gu, const float* __restrict__ gv,
                                                          const float* __restrict__ gw, const float* __restrict__ gp,
                                                          float* __restrict__ b_hi, float* __restrict__ b_lo,
                                                          Scalars* sc, double* partials, int nblocks) {
    __shared__ double sh[8 * 1];
    Acc acc;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const float inv_h = 1.0f / h;
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        df s = {0.0f, 0.0f};
        if (cls[i] == 1) {
            const Nbr nb = neighbours(g, x, y, z);
            const float ai = alpha[i];
            if (nb.xm >= 0 && cls[nb.xm] != 0) {
                float gf = gu[x + (nx + 1) * (y + ny * z)];
                if (x == 0) gf += gu[nx + (nx + 1) * (y + ny * z)];
                s = df_add(s, two_prod(-mobility_of(mob, alpha[nb.xm], ai, nb.xm, i) * inv_h, gf));
            }
            if (nb.xp >= 0 && cls[nb.xp] != 0) {
                const int hx = x + 1 == nx ? 0 : x + 1;
                float gf = gu[hx + (nx + 1) * (y + ny * z)];
                if (hx == 0) gf += gu[nx + (nx + 1) * (y + ny * z)];
                s = df_add(s, two_prod(mobility_of(mob, ai, alpha[nb.xp], i, nb.xp) * inv_h, gf));
            }
            if (nb.ym >= 0 && cls[nb.ym] != 0) {
                float gf = gv[x + nx * (y + (ny + 1) * z)];
                if (y == 0) gf += gv[x + nx * (ny + (ny + 1) * z)];
                s = df_add(s, two_prod(-mobility_of(mob, alpha[nb.ym], ai, nb.ym, i) * inv_h, gf));
            }
            if (nb.yp >= 0 && cls[nb.yp] != 0) {
                const int hy = y + 1 == ny ? 0 : y + 1;
                float gf = gv[x + nx * (hy + (ny + 1) * z)];
                if (hy == 0) gf += gv[x + nx * (ny + (ny + 1) * z)];
                s = df_add(s, two_prod(mobility_of(mob, ai, alpha[nb.yp], i, nb.yp) * inv_h, gf));
            }
            if (nb.zm >= 0 && cls[nb.zm] != 0) {
                float gf = gw[x + nx * (y + ny * z)];
                if (z == 0) gf += gw[x + nx * (y + ny * nz)];
                s = df_add(s, two_prod(-mobility_of(mob, alpha[nb.zm], ai, nb.zm, i) * inv_h, gf));
            }
            if (nb.zp >= 0 && cls[nb.zp] != 0) {
                const int hz = z + 1 == nz ? 0 : z + 1;
                float gf = gw[x + nx * (y + ny * hz)];
                if (hz == 0) gf += gw[x + nx * (y + ny * nz)];
                s = df_add(s, two_prod(mobility_of(mob, ai, alpha[nb.zp], i, nb.zp) * inv_h, gf));
            } else if (nb.zp < 0 && outlet && z == nz - 1) {
                s = df_add(s, two_prod(gtop[x + nx * y] * inv_h, gw[x + nx * (y + ny * nz)]));
            }
            if (gp) s = df_add(s, two_prod(p_scale, gp[i]));
        }
        b_hi[i] = s.hi;
        b_lo[i] = s.lo;
        acc.add_prod(s.hi, s.hi);
    }
    double v1[1] = {acc.total()};
    block_sum<1>(v1, sh);
    if (store_partials_is_last<1>(v1, partials, nblocks, &sc->ticket[0])) {
        double tot[1];
        finish_partials<1>(tot, partials, nblocks, sh, &sc->ticket[0]);
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            sc->bb = tot[0];
            if (!isfinite(tot[0])) sc->nonfinite = 1;
        }
    }
}

// g_u* = g_u (folded) - h D^T psi on open faces; 0 on closed and duplicate faces.
__global__ void __launch_bounds__(TILE_THREADS) k_adj_correct(Grid3 g, int outlet, float h,
                                                              const uint8_t* __restrict__ cls,
                                                              const float* __restrict__ sh_, const float* __restrict__ sl_,
                                                              const float* __restrict__ gu,
                                                              const float* __restrict__ gv,
                                                              const float* __restrict__ gw, float* __restrict__ ou,
                                                              float* __restrict__ ov, float* __restrict__ ow) {
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        const Nbr nb = neighbours(g, x, y, z);
        const uint8_t ci = cls[i];
        const df si = {sh_[i], sl_[i]};
        {
            const int f = x + (nx + 1) * (y + ny * z), fd = nx + (nx + 1) * (y + ny * z);
            float out = 0.0f;
            if (nb.xm >= 0 && ci != 0 && cls[nb.xm] != 0) {
                float gf = gu[f];
                if (x == 0) gf += gu[fd];
                out = gf + h * df_to_f(df_sub(si, df{sh_[nb.xm], sl_[nb.xm]}));
            }
            ou[f] = out;
            if (x == nx - 1) ou[fd] = 0.0f;
        }
        {
            const int f = x + nx * (y + (ny + 1) * z), fd = x + nx * (ny + (ny + 1) * z);
            float out = 0.0f;
            if (nb.ym >= 0 && ci != 0 && cls[nb.ym] != 0) {
                float gf = gv[f];
                if (y == 0) gf += gv[fd];
                out = gf + h * df_to_f(df_sub(si, df{sh_[nb.ym], sl_[nb.ym]}));
            }
            ov[f] = out;
            if (y == ny - 1) ov[fd] = 0.0f;
        }
        {
            const int f = x + nx * (y + ny * z), fd = x + nx * (y + ny * nz);
            float out = 0.0f;
            if (nb.zm >= 0 && ci != 0 && cls[nb.zm] != 0) {
                float gf = gw[f];
                if (z == 0 && (g.periodic & 4)) gf += gw[fd];
                out = gf + h * df_to_f(df_sub(si, df{sh_[nb.zm], sl_[nb.zm]}));
            }
            ow[f] = out;
            if (z == nz - 1) {
                float top = 0.0f;
                if (outlet && !(g.periodic & 4) && ci != 0) top = gw[fd] - h * df_to_f(si);
                ow[fd] = top;
            }
        }
    }
}

// u* = u + dt f / rho_face on open faces (closed faces copied through).
__device__ __forceinline__ double face_rho(float aL, float aR, float rho_l, float rho_air) {
    return 0.5 * ((double)rho_of(aL, rho_l, rho_air) + (double)rho_of(aR, rho_l, rho_air));
}
__global__ void __launch_bounds__(TILE_THREADS) k_add_force(Grid3 g, int outlet, float rho_l, float rho_air,
                                                            const uint8_t* __restrict__ cls,
                                                            const float* __restrict__ alpha, const float* u,
                                                            const float* v, const float* w,
                                                            const float* __restrict__ fu,
                                                            const float* __restrict__ fv,
                                                            const float* __restrict__ fw, float dt, float* su,
                                                            float* sv, float* sw) {
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const double dtd = (double)dt;
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        const Nbr nb = neighbours(g, x, y, z);
        const uint8_t ci = cls[i];
        {
            const int f = x + (nx + 1) * (y + ny * z);
            float out = u[f];
            if (nb.xm >= 0 && ci != 0 && cls[nb.xm] != 0)
                out = (float)((double)u[f] + dtd * (double)fu[f] / face_rho(alpha[nb.xm], alpha[i], rho_l, rho_air));
            su[f] = out;
            if (x == nx - 1) su[nx + (nx + 1) * (y + ny * z)] = u[nx + (nx + 1) * (y + ny * z)];
        }
        {
            const int f = x + nx * (y + (ny + 1) * z);
            float out = v[f];
            if (nb.ym >= 0 && ci != 0 && cls[nb.ym] != 0)
                out = (float)((double)v[f] + dtd * (double)fv[f] / face_rho(alpha[nb.ym], alpha[i], rho_l, rho_air));
            sv[f] = out;
            if (y == ny - 1) sv[x + nx * (ny + (ny + 1) * z)] = v[x + nx * (ny + (ny + 1) * z)];
        }
        {
            const int f = x + nx * (y + ny * z);
            float out = w[f];
            if (nb.zm >= 0 && ci != 0 && cls[nb.zm] != 0)
                out = (float)((double)w[f] + dtd * (double)fw[f] / face_rho(alpha[nb.zm], alpha[i], rho_l, rho_air));
            sw[f] = out;
            if (z == nz - 1) {
                const int ft = x + nx * (y + ny * nz);
                float top = w[ft];
                if (outlet && !(g.periodic & 4) && ci != 0)
                    top = (float)((double)w[ft] + dtd * (double)fw[ft] / (double)rho_of(alpha[i], rho_l, rho_air));
                sw[ft] = top;
            }
        }
    }
}
// g_f += dt / rho_face * lambda on open (canonical) faces.
__global__ void __launch_bounds__(TILE_THREADS) k_force_grad(Grid3 g, int outlet, float rho_l, float rho_air,
                                                             const uint8_t* __restrict__ cls,
                                                             const float* __restrict__ alpha,
                                                             const float* __restrict__ lu,
                                                             const float* __restrict__ lv,
                                                             const float* __restrict__ lw, float dt,
                                                             double* __restrict__ gu, double* __restrict__ gv,
                                                             double* __restrict__ gw) {
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const double dtd = (double)dt;
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        const Nbr nb = neighbours(g, x, y, z);
        const uint8_t ci = cls[i];
        if (nb.xm >= 0 && ci != 0 && cls[nb.xm] != 0) {
            const int f = x + (nx + 1) * (y + ny * z);
            gu[f] += dtd / face_rho(alpha[nb.xm], alpha[i], rho_l, rho_air) * (double)lu[f];
        }
        if (nb.ym >= 0 && ci != 0 && cls[nb.ym] != 0) {
            const int f = x + nx * (y + (ny + 1) * z);
            gv[f] += dtd / face_rho(alpha[nb.ym], alpha[i], rho_l, rho_air) * (double)lv[f];
        }
        if (nb.zm >= 0 && ci != 0 && cls[nb.zm] != 0) {
            const int f = x + nx * (y + ny * z);
            gw[f] += dtd / face_rho(alpha[nb.zm], alpha[i], rho_l, rho_air) * (double)lw[f];
        }
        if (z == nz - 1 && outlet && !(g.periodic & 4) && ci != 0) {
            const int ft = x + nx * (y + ny * nz);
            gw[ft] += dtd / (double)rho_of(alpha[i], rho_l, rho_air) * (double)lw[ft];
        }
    }
}
// J = sum over outlet faces of w^2 (into sc->objective, or added to it when
// `accumulate`); seed_w = 2 w there (added to seed_w when `add_seed`).
__global__ void __launch_bounds__(TILE_THREADS) k_outlet_objective(Grid3 g, const float* __restrict__ w,
                                                                   float* __restrict__ seed_w, Scalars* sc,
                                                                   double* partials, int nblocks, int accumulate,
                                                                   int add_seed) {
    __shared__ double sh[8 * 1];
    double acc[1] = {0.0};
    const int x = blockIdx.x * TX + threadIdx.x;
    const int y = blockIdx.y * TY + threadIdx.y;
    if (x < g.nx && y < g.ny && blockIdx.z == 0) {
        const int ft = x + g.nx * (y + g.ny * g.nz);
        const double wz = w[ft];
        acc[0] = wz * wz;
        if (seed_w) seed_w[ft] = add_seed ? seed_w[ft] + (float)(2.0 * wz) : (float)(2.0 * wz);
    }
    block_sum<1>(acc, sh);
    if (store_partials_is_last<1>(acc, partials, nblocks, &sc->ticket[6])) {
        double tot[1];
        finish_partials<1>(tot, partials, nblocks, sh, &sc->ticket[6]);
        if (threadIdx.x == 0 && threadIdx.y == 0) sc->objective = accumulate ? sc->objective + tot[0] : tot[0];
    }
}

// ----------------------------------------------------------- launchers
Launch tile_launch(int nx, int ny, int nz, int periodic, int target_blocks) {
    Launch L;
    L.block = dim3(TX, TY, 1);
    const int gx = (nx + TX - 1) / TX, gy = (ny + TY - 1) / TY;
    const int tiles = gx * gy;
    int zc = (target_blocks + tiles - 1) / tiles;
    if (zc > nz) zc = nz;
    if (zc < 1) zc = 1;
    int zper = (nz + zc - 1) / zc;
    if ((zper & 1) && zper < nz) zper += 1;  // even runs: restriction pairs planes within a block
    zc = (nz + zper - 1) / zper;
    while ((long long)tiles * zc > MAX_REDUCE_BLOCKS && zper < nz) {
        zper *= 2;
        zc = (nz + zper - 1) / zper;
    }
    L.grid = dim3(gx, gy, zc);
    L.g.nx = nx;
    L.g.ny = ny;
    L.g.nz = nz;
    L.g.periodic = periodic;
    L.g.zper = zper;
    L.nblocks = tiles * zc;
    return L;
}

void launch_coefficients(const Launch& L, const Fields& F, cudaStream_t s) {
    k_coefficients<<<L.grid, L.block, 0, s>>>(L.g, F.outlet, F.alpha, F.cls, F.mob, F.coef, F.coef_lo,
                                              F.coef_lo_kind, F.gtop);
}
void launch_init_scalars(Scalars* sc, double tol2, double abs_floor, double inner_floor2, int max_total,
                         cudaStream_t s) {
    k_init_scalars<<<1, 1, 0, s>>>(sc, tol2, abs_floor, inner_floor2, max_total);
}
void launch_set_sigma(Scalars* sc, float sigma, cudaStream_t s) { k_set_sigma<<<1, 1, 0, s>>>(sc, sigma); }
// Measurement of the pipelined kernels in isolation: a mid-pass state with
// zero step lengths (the kernels do all their loads, arithmetic and stores;
// the fields keep their values).
__global__ void k_profile_reset(Scalars* sc, int no_stop) {
    sc->sigma = sc->inv_sigma = sc->inv_sigma_z = 1.0f;
    sc->converged = 0;
    sc->first = 0;
    sc->alpha_f = sc->beta_f = 0.0f;
    if (no_stop) {  // repeated launches of one kernel never meet the stop test
        sc->rr_target = -1.0;
        sc->max_total = 0x7fffffff;
    }
}
void launch_profile_reset(Scalars* sc, cudaStream_t s, bool no_stop) { k_profile_reset<<<1, 1, 0, s>>>(sc, no_stop ? 1 : 0); }
void launch_rhs(const Launch& L, const Fields& F, const float* u, const float* v, const float* w, cudaStream_t s,
                bool start_pass) {
    k_rhs<<<L.grid, L.block, 0, s>>>(L.g, F.outlet, F.h, F.cls, u, v, w, F.b_hi, F.b_lo, F.r, F.e, start_pass ? 1 : 0,
                                     F.sc, F.partials, L.nblocks, F.n_active);
}
void launch_residual(const Launch& L, const Fields& F, const float* x_hi, const float* x_lo, cudaStream_t s) {
    k_residual<<<L.grid, L.block, 0, s>>>(L.g, F.coef, F.b_hi, F.b_lo, x_hi, x_lo, F.r, F.e, F.sc, F.partials,
                                          L.nblocks, F.n_active);
}
void launch_spmv_pq(const Launch& L, const Fields& F, cudaStream_t s) {
    k_spmv_pq<<<L.grid, L.block, 0, s>>>(L.g, F.coef, F.p, F.q, F.sc, F.partials, L.nblocks);
}
static int flat_blocks(long long n) {
    const long long want = (n / 4 + 255) / 256;
    return (int)(want < 1 ? 1 : (want < FLAT_BLOCKS ? want : FLAT_BLOCKS));
}
void launch_update(const Launch& L, const Fields& F, cudaStream_t s) {
    const long long n = L.g.n();
    const int nb = flat_blocks(n);
    k_update<<<nb, 256, 0, s>>>(n, F.e, F.r, F.p, F.q, F.sc, F.partials, nb, F.n_active);
}
void launch_dot_rz(const Launch& L, const Fields& F, int init, cudaStream_t s) {
    const long long n = L.g.n();
    const int nb = flat_blocks(n);
    k_dot_rz<<<nb, 256, 0, s>>>(n, F.r, F.z, F.p, init, F.sc, F.partials, nb);
}
void launch_search(const Launch& L, const Fields& F, cudaStream_t s) {
    const long long n = L.g.n();
    k_search<<<flat_blocks(n), 256, 0, s>>>(n, F.z, F.p, F.sc);
}
void launch_accumulate(const Launch& L, const Fields& F, float* x_hi, float* x_lo, cudaStream_t s) {
    k_accumulate<<<L.grid, L.block, 0, s>>>(L.g, x_hi, x_lo, F.e);
}
void launch_accumulate_pipelined(const Launch& L, float* x_hi, float* x_lo, const float* x, const float* p0,
                                 const float* p1, const Scalars* sc, cudaStream_t s) {
    k_accumulate_pipelined<<<L.grid, L.block, 0, s>>>(L.g, x_hi, x_lo, x, p0, p1, sc);
}
void launch_to_double(const float* hi, const float* lo, double* out, long long n, cudaStream_t s) {
    k_to_double<<<152 * 4, 256, 0, s>>>(hi, lo, out, n);
}
void launch_correct(const Launch& L, const Fields& F, const float* ph, const float* pl, const float* us,
                    const float* vs, const float* ws, float* uo, float* vo, float* wo, float* po, float dt,
                    cudaStream_t s) {
    const float p_scale = (float)((double)F.rho_l / (double)dt);
    k_correct<<<L.grid, L.block, 0, s>>>(L.g, F.outlet, F.h, F.mob, p_scale, F.cls, F.alpha, F.gtop, ph,
                                         pl, us, vs, ws, uo, vo, wo, po);
}
void launch_divergence(const Launch& L, const Fields& F, const float* u, const float* v, const float* w,
                       cudaStream_t s) {
    k_divergence<<<L.grid, L.block, 0, s>>>(L.g, F.h, F.cls, u, v, w, F.sc, F.partials, L.nblocks);
}
void launch_apply(const Launch& L, const Fields& F, const float* x, float* y, cudaStream_t s) {
    k_apply<<<L.grid, L.block, 0, s>>>(L.g, F.coef, x, y);
}
void launch_scale(const Launch& L, const float* in, float* out, float scale, const Scalars* sc, cudaStream_t s) {
    k_scale<<<L.grid, L.block, 0, s>>>(L.g, in, out, scale, sc);
}
void launch_adj_rhs(const Launch& L, const Fields& F, const float* gu, const float* gv, const float* gw,
                    const float* gp, float dt, cudaStream_t s) {
    const float p_scale = (float)((double)F.rho_l / (double)dt);
    k_adj_rhs<<<L.grid, L.block, 0, s>>>(L.g, F.outlet, F.h, F.mob, p_scale, F.cls, F.alpha, F.gtop, gu,
                                         gv, gw, gp, F.b_hi, F.b_lo, F.sc, F.partials, L.nblocks);
}
void launch_adj_correct(const Launch& L, const Fields& F, const float* psi_hi, const float* psi_lo, const float* gu,
                        const float* gv, const float* gw, float* ou, float* ov, float* ow, cudaStream_t s) {
    k_adj_correct<<<L.grid, L.block, 0, s>>>(L.g, F.outlet, F.h, F.cls, psi_hi, psi_lo, gu, gv, gw, ou, ov, ow);
}
void launch_add_force(const Launch& L, const Fields& F, const float* u, const float* v, const float* w,
                      const float* fu, const float* fv, const float* fw, float dt, float* su, float* sv, float* sw,
                      cudaStream_t s) {
    k_add_force<<<L.grid, L.block, 0, s>>>(L.g, F.outlet, F.rho_l, F.rho_air, F.cls, F.alpha, u, v, w, fu, fv, fw, dt,
                                           su, sv, sw);
}
void launch_force_grad(const Launch& L, const Fields& F, const float* lu, const float* lv, const float* lw, float dt,
                       double* gu, double* gv, double* gw, cudaStream_t s) {
    k_force_grad<<<L.grid, L.block, 0, s>>>(L.g, F.outlet, F.rho_l, F.rho_air, F.cls, F.alpha, lu, lv, lw, dt, gu, gv,
                                            gw);
}
void launch_outlet_objective(const Launch& L, const Fields& F, const float* w, float* seed_w, cudaStream_t s,
                             bool accumulate, bool add_seed) {
    dim3 grid(L.grid.x, L.grid.y, 1);
    k_outlet_objective<<<grid, L.block, 0, s>>>(L.g, w, seed_w, F.sc, F.partials, (int)(grid.x * grid.y),
                                                accumulate ? 1 : 0, add_seed ? 1 : 0);
}

}  // namespace mhdproj
