// fine_kernels.cu -- the finest-level stencil kernels with shared-memory
// plane staging.
//
// A block of 32 x 8 threads owns a 64 x 8 (x, y) tile -- each thread an
// x-pair of cells -- and marches it along z.  A ring of plane slots in
// shared memory holds, per plane: the vector tile with its halo (columns
// x0-2 .. x0+65, rows y0-1 .. y0+8), the coefficient records of the tile plus
// its +x column and +y row (the high faces), and the right-hand side of the
// tile.  Planes are fetched with 8- and 16-byte cp.async two planes ahead of
// the plane being computed, so loads stay in flight while warps compute from
// shared memory, and every value is read from HBM once per block (halo
// re-reads hit L2).  Outside a closed boundary copies are zero-filled, which
// is the zero coefficient of a wall face; periodic axes wrap the source.
// The kernels need an even nx (cell pairs never straddle the domain edge);
// other grids use the per-cell kernels of mg_kernels.cu / gb300_kernels.cu.
//
// In a red-black half-step exactly one cell of each pair has the colour being
// updated, so every lane works.  Cells of one colour are never neighbours of
// each other (odd periodic extents use the out-of-place variant), so the
// staged snapshots are exactly the values each update reads.
#include <algorithm>
#include <cmath>
#include <type_traits>

#include "kernels.h"
#include "staged.cuh"

namespace mhdproj {

namespace {
constexpr int PX = 2 * TX;               // cells per tile row
constexpr int EW = PX + 4, EH = TY + 2;  // vector tile: x0-2 .. x0+PX+1 (pairs)
constexpr int EP = EW / 2;               // float2 pairs per vector row
constexpr int CW = PX + 2, CH = TY + 1;  // coefficient tile: x0 .. x0+PX (+1 pad)
// Ring depth: planes z-1 .. z+PF.  Two planes ahead with five blocks per SM
// keeps about 100 KB of copies in flight per SM, twice what the HBM latency
// needs, while leaving room for 40 resident warps.
template <int CK> struct Depth {
    static constexpr int NSLOT = 4;
    static constexpr int PF = NSLOT - 2;
};

using namespace staged;
template <int PF>
__device__ __forceinline__ void cp_wait_pf() { cp_wait<PF - 1>(); }
__device__ __forceinline__ void cp_wait0() { cp_wait<0>(); }

template <int CK>
struct Ring {
    using CT = typename CoefStore<CK>::T;
    static constexpr int NSLOT = Depth<CK>::NSLOT;
    float e[NSLOT][EH][EW];
    CT c[NSLOT][CH][CW];
    float r[NSLOT][TY][PX];
};

// A thread's share of the plane copies, resolved once per block.  Vector
// tile: 10 rows x 34 float2 pairs; coefficients: 9 rows x 65 records (16-byte
// FP32 records) or 9 rows x (32 record pairs + 1 record) (8-byte records);
// right-hand side: 8 rows x 32 float2.
template <int CK>
struct Fetcher {
    static constexpr int NE = EH * EP;
    static constexpr int CPR = (CK == 0) ? PX + 1 : TX + 1;
    static constexpr int NC = CH * CPR;
    int eoff[2], coff[3], roff;
    short edst[2], cdst[3];
    unsigned char csize[3];  // 0 none, 1 one record, 2 two records
    bool eok[2], cok[3], rok;
    long long sxy;
    int nz;
    bool pz;

    __device__ __forceinline__ Fetcher(const Grid3& g, int x0, int y0) {
        const int t = threadIdx.x + TX * threadIdx.y;
        sxy = (long long)g.nx * g.ny;
        nz = g.nz;
        pz = (g.periodic & 4) != 0;
        const bool px = g.periodic & 1, py = g.periodic & 2;
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const int k = t + j * TILE_THREADS;
            eok[j] = false;
            eoff[j] = 0;
            edst[j] = -1;
            if (k < NE) {
                const int ty = k / EP, pi = k - ty * EP;
                bool okx, oky;
                const int sx = axis_src(x0 - 2 + 2 * pi, g.nx, px, &okx);
                const int sy = axis_src(y0 - 1 + ty, g.ny, py, &oky);
                eok[j] = okx && oky;
                eoff[j] = eok[j] ? sx + g.nx * sy : 0;
                edst[j] = (short)(ty * EW + 2 * pi);
            }
        }
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const int k = t + j * TILE_THREADS;
            cok[j] = false;
            coff[j] = 0;
            cdst[j] = 0;
            csize[j] = 0;
            if (k < NC) {
                const int ty = k / CPR, ci = k - ty * CPR;
                const int cx = (CK == 0) ? ci : (ci < TX ? 2 * ci : PX);
                bool okx, oky;
                const int sx = axis_src(x0 + cx, g.nx, px, &okx);
                const int sy = axis_src(y0 + ty, g.ny, py, &oky);
                cok[j] = okx && oky;
                coff[j] = cok[j] ? sx + g.nx * sy : 0;
                cdst[j] = (short)(ty * CW + cx);
                csize[j] = (CK != 0 && ci < TX) ? 2 : 1;
            }
        }
        const int rx = x0 + 2 * threadIdx.x, ry = y0 + threadIdx.y;
        rok = rx < g.nx && ry < g.ny;
        roff = rok ? rx + g.nx * ry : 0;
    }

    template <bool WANT_E, bool WANT_R>
    __device__ __forceinline__ void fetch(Ring<CK>& R, int zz, int slot, const float* ev,
                                          const typename CoefStore<CK>::T* coef, const float* rv) const {
        bool okz;
        const int sz = axis_src(zz, nz, pz, &okz);
        const long long plane = (long long)sz * sxy;
        if (WANT_E) {
            float* dst = &R.e[slot][0][0];
#pragma unroll
            for (int j = 0; j < 2; j++)
                if (edst[j] >= 0) {
                    const bool ok = eok[j] && okz;
                    cp_async8(dst + edst[j], ev + (ok ? plane + eoff[j] : 0), ok);
                }
        }
        auto* cd = &R.c[slot][0][0];
#pragma unroll
        for (int j = 0; j < 3; j++)
            if (csize[j]) {
                const bool ok = cok[j] && okz;
                const auto* src = coef + (ok ? plane + coff[j] : 0);
                if (CK == 0 || csize[j] == 2) cp_async16(cd + cdst[j], src, ok);
                else cp_async8(cd + cdst[j], src, ok);
            }
        if (WANT_R) {
            const bool ok = rok && zz >= 0 && zz < nz;
            cp_async8(&R.r[slot][threadIdx.y][2 * threadIdx.x], rv + (ok ? plane + roff : 0), ok);
        }
    }
};

template <int CK>
__device__ __forceinline__ int slot_of(int zz, int z0) { return (zz - z0 + 1) & (Depth<CK>::NSLOT - 1); }

// Prologue: planes z0-1 .. z0+PF-1 in flight, one commit group each (z0-1
// and z0 together).
template <bool WANT_E, bool WANT_R, int CK>
__device__ __forceinline__ void prologue(const Fetcher<CK>& F, Ring<CK>& R, int z0, int z1, const float* ev,
                                         const typename CoefStore<CK>::T* coef, const float* rv) {
    constexpr int PF = Depth<CK>::PF;
    F.template fetch<WANT_E, WANT_R>(R, z0 - 1, slot_of<CK>(z0 - 1, z0), ev, coef, rv);
    F.template fetch<WANT_E, WANT_R>(R, z0, slot_of<CK>(z0, z0), ev, coef, rv);
    cp_commit();
#pragma unroll
    for (int k = 1; k < PF; k++) {
        if (z0 + k <= z1) F.template fetch<WANT_E, WANT_R>(R, z0 + k, slot_of<CK>(z0 + k, z0), ev, coef, rv);
        cp_commit();
    }
}
// Next plane in flight, then wait until planes up to z+1 have landed.
template <bool WANT_E, bool WANT_R, int CK>
__device__ __forceinline__ void advance(const Fetcher<CK>& F, Ring<CK>& R, int z, int z0, int z1, const float* ev,
                                        const typename CoefStore<CK>::T* coef, const float* rv) {
    constexpr int PF = Depth<CK>::PF;
    if (z + PF <= z1) F.template fetch<WANT_E, WANT_R>(R, z + PF, slot_of<CK>(z + PF, z0), ev, coef, rv);
    cp_commit();
    cp_wait_pf<PF>();
    __syncthreads();
}
}  // namespace

// --------------------------------------------------------------- SpMV
__global__ void __launch_bounds__(TILE_THREADS) k_spmv_staged(Grid3 g, const float4* __restrict__ coef,
                                                              const float* __restrict__ p, float* __restrict__ q,
                                                              Scalars* sc, double* partials, int nblocks) {
    if (sc->converged) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto& R = *reinterpret_cast<Ring<0>*>(smem_raw);
    __shared__ double sh[8];
    const int x0 = blockIdx.x * PX, y0 = blockIdx.y * TY;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x = x0 + 2 * tx, y = y0 + ty;
    const int z0 = blockIdx.z * g.zper, z1 = min(g.nz, z0 + g.zper);
    const bool inside = x < g.nx && y < g.ny;
    Acc acc;
    const Fetcher<0> F(g, x0, y0);
    prologue<true, false>(F, R, z0, z1, p, coef, nullptr);
    for (int z = z0; z < z1; z++) {
        advance<true, false>(F, R, z, z0, z1, p, coef, nullptr);
        if (inside) {
            const int s = slot_of<0>(z, z0), sm = slot_of<0>(z - 1, z0), sp = slot_of<0>(z + 1, z0);
            const float* er = &R.e[s][ty + 1][0];
            float qv[2];
#pragma unroll
            for (int k = 0; k < 2; k++) {
                const int cx = 2 * tx + k, ex = cx + 2;
                const float4 cc = R.c[s][ty][cx];
                const float bxh = R.c[s][ty][cx + 1].x, byh = R.c[s][ty + 1][cx].y, bzh = R.c[sp][ty][cx].z;
                const float pc = er[ex];
                float v = cc.w * pc;
                v = fmaf(cc.x, pc - er[ex - 1], v);
                v = fmaf(bxh, pc - er[ex + 1], v);
                v = fmaf(cc.y, pc - R.e[s][ty][ex], v);
                v = fmaf(byh, pc - R.e[s][ty + 2][ex], v);
                v = fmaf(cc.z, pc - R.e[sm][ty + 1][ex], v);
                v = fmaf(bzh, pc - R.e[sp][ty + 1][ex], v);
                qv[k] = v;
                acc.add_prod(pc, v);
            }
            *reinterpret_cast<float2*>(q + x + (long long)g.nx * (y + (long long)g.ny * z)) = make_float2(qv[0], qv[1]);
        }
        __syncthreads();
    }
    cp_wait0();
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

// ------------------------------------------------- search step + SpMV
// Pipelined CG step: the new search direction p = z / sigma_z + beta p_old is
// formed plane by plane over the tile with its 1-cell halo (halo values are
// recomputed by the neighbouring tiles from the same inputs), written for the
// tile, and q = A p, p . q follow one plane behind.  The solution update of
// the previous step, x += alpha_prev p_old, rides along (the residual update
// happens in the pre-smoothing pass).  At the start of a CG pass p = z / sigma_z
// and x is left alone.  Staged vector rows span x0-4 .. x0+67 (16-byte
// copies of four cells; nx must be a multiple of 4).
namespace {
constexpr int SW = PX + 8;             // 72 staged columns: x0-4 .. x0+67
constexpr int SG = SW / 4;             // 18 four-cell groups per row
constexpr int NSV = EH * SG;           // 180 vector copies per plane
constexpr int NSX = TY * (PX / 4);     // 128 copies of the tile's x
constexpr int NSC = CH * (PX + 1);     // 585 coefficient records
}  // namespace
// A step forms p on plane zA and q on plane zA-1 and stages plane zA+1;
// ring sizes 2 and 4 let the z loop unroll four times with compile-time slots.
struct SearchRing {
    float4 c[4][CH][CW];   // planes zA-2 .. zA+1 (x0 .. x0+64, y0 .. y0+8)
    float zt[2][EH][SW];   // planes zA .. zA+1 (y0-1 .. y0+8)
    float po[2][EH][SW];
    float xs[2][TY][PX];
    float pn[4][EH][SW];   // planes zA-3 .. zA
};

__global__ void __launch_bounds__(TILE_THREADS) k_search_spmv(Grid3 g, const float4* __restrict__ coef,
                                                              const float* __restrict__ zv,
                                                              const float* __restrict__ p_old,
                                                              float* __restrict__ p_new, float* __restrict__ xs,
                                                              float* __restrict__ q, Scalars* sc, double* partials,
                                                              int nblocks, int pidx_new) {
    if (sc->converged) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto& S = *reinterpret_cast<SearchRing*>(smem_raw);
    __shared__ double sh[8];
    const bool first = sc->first != 0;
    const float is = sc->inv_sigma_z, bt = sc->beta_f, ap = sc->alpha_f;
    const int x0 = blockIdx.x * PX, y0 = blockIdx.y * TY;
    const int tx = threadIdx.x, ty = threadIdx.y, t = tx + TX * ty;
    const int z0 = blockIdx.z * g.zper, z1 = min(g.nz, z0 + g.zper);
    const bool px = g.periodic & 1, py = g.periodic & 2, pz = (g.periodic & 4) != 0;
    const long long sxy = (long long)g.nx * g.ny;
    // copy descriptors
    int voff = 0, xoff = 0, coff[3] = {0, 0, 0};
    short vdst = -1, xdst = -1, cdst[3] = {-1, -1, -1};
    bool vok = false, xok = false, cok[3] = {false, false, false};
    if (t < NSV) {
        const int row = t / SG, gi = t - row * SG;
        bool okx, oky;
        const int sx = axis_src(x0 - 4 + 4 * gi, g.nx, px, &okx);
        const int sy = axis_src(y0 - 1 + row, g.ny, py, &oky);
        vok = okx && oky;
        voff = vok ? sx + g.nx * sy : 0;
        vdst = (short)(row * SW + 4 * gi);
    }
    if (t < NSX) {
        const int row = t / (PX / 4), gi = t - row * (PX / 4);
        const int gx = x0 + 4 * gi, gy = y0 + row;
        xok = gx < g.nx && gy < g.ny;
        xoff = xok ? gx + g.nx * gy : 0;
        xdst = (short)(row * PX + 4 * gi);
    }
#pragma unroll
    for (int u = 0; u < 3; u++) {
        const int k = t + u * TILE_THREADS;
        if (k < NSC) {
            const int row = k / (PX + 1), cx = k - row * (PX + 1);
            bool okx, oky;
            const int sx = axis_src(x0 + cx, g.nx, px, &okx);
            const int sy = axis_src(y0 + row, g.ny, py, &oky);
            cok[u] = okx && oky;
            coff[u] = cok[u] ? sx + g.nx * sy : 0;
            cdst[u] = (short)(row * CW + cx);
        }
    }
    auto fetch = [&](int zz, int s2, int s4) {
        bool okz;
        const int sz = axis_src(zz, g.nz, pz, &okz);
        const long long plane = (long long)sz * sxy;
        if (vdst >= 0) {
            const bool ok = vok && okz;
            const long long o = ok ? plane + voff : 0;
            cp_async16(&S.zt[s2][0][0] + vdst, zv + o, ok);
            if (!first) cp_async16(&S.po[s2][0][0] + vdst, p_old + o, ok);
        }
        if (!first && xdst >= 0) {
            const bool ok = xok && zz >= 0 && zz < g.nz;
            cp_async16(&S.xs[s2][0][0] + xdst, xs + (ok ? plane + xoff : 0), ok);
        }
#pragma unroll
        for (int u = 0; u < 3; u++)
            if (cdst[u] >= 0) {
                const bool ok = cok[u] && okz;
                cp_async16(&S.c[s4][0][0] + cdst[u], coef + (ok ? plane + coff[u] : 0), ok);
            }
    };
    // pair tasks over x0-2 .. x0+65, y0-1 .. y0+8: flat offsets, tile pairs'
    // in-plane offsets (-1 off the tile) and their x staging offsets
    constexpr int NT = EH * EP;
    int toff[2] = {-1, -1}, town[2] = {-1, -1}, txo[2] = {0, 0};
#pragma unroll
    for (int u = 0; u < 2; u++) {
        const int k = t + u * TILE_THREADS;
        if (k < NT) {
            const int row = k / EP, pc = k - row * EP;
            toff[u] = row * SW + 2 + 2 * pc;
            const int gx = x0 - 2 + 2 * pc, gy = y0 - 1 + row;
            if (row >= 1 && row <= TY && pc >= 1 && pc <= TX && gx < g.nx && gy < g.ny) {
                town[u] = gx + g.nx * gy;
                txo[u] = (row - 1) * PX + 2 * pc - 2;
            }
        }
    }
    // q stage: thread tx takes cells x0+tx and x0+tx+32 of row ty, so every
    // shared-memory read of a warp is unit-stride (adjacent cell pairs made
    // the float4 records two-way and their neighbour-face lanes eight-way
    // bank conflicts)
    Acc acc;
    const int oy = y0 + ty;
    const bool own_row = oy < g.ny;
    const int oo = (ty + 1) * SW + 4 + tx, co = ty * CW + tx;
    const long long og = x0 + tx + (long long)g.nx * oy;
    auto step = [&](auto ph, int zA) {
        constexpr int P = decltype(ph)::value;
        fetch(zA + 1, (P + 1) & 1, (P + 1) & 3);
        cp_commit();
        cp_wait<1>();
        __syncthreads();
        {
            const float* ZT = &S.zt[P & 1][0][0];
            const float* PO = &S.po[P & 1][0][0];
            const float* XS = &S.xs[P & 1][0][0];
            float* PN = &S.pn[P][0][0];
            const bool zin = zA >= z0 && zA < z1;
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const int o = toff[u];
                if (o < 0) break;
                const float2 zz = *reinterpret_cast<const float2*>(ZT + o);
                float2 pn, po = make_float2(0.f, 0.f);
                if (first) {
                    pn = make_float2(zz.x * is, zz.y * is);
                } else {
                    po = *reinterpret_cast<const float2*>(PO + o);
                    pn = make_float2(fmaf(bt, po.x, zz.x * is), fmaf(bt, po.y, zz.y * is));
                }
                *reinterpret_cast<float2*>(PN + o) = pn;
                if (zin && town[u] >= 0) {
                    const long long i0 = town[u] + sxy * zA;
                    *reinterpret_cast<float2*>(p_new + i0) = pn;
                    if (!first) {
                        const float2 xv = *reinterpret_cast<const float2*>(XS + txo[u]);
                        *reinterpret_cast<float2*>(xs + i0) = make_float2(fmaf(ap, po.x, xv.x), fmaf(ap, po.y, xv.y));
                    }
                }
            }
        }
        __syncthreads();
        const int z = zA - 1;
        if (z >= z0 && z < z1 && own_row) {
            const float* Pc = &S.pn[(P + 3) & 3][0][0];
            const float* PM = &S.pn[(P + 2) & 3][0][0];
            const float* PP = &S.pn[P][0][0];
            const float4* C = &S.c[(P + 3) & 3][0][0];
            const float4* CN = &S.c[P][0][0];
#pragma unroll
            for (int k = 0; k < 2; k++) {
                if (x0 + tx + 32 * k >= g.nx) break;
                const int o = oo + 32 * k, c = co + 32 * k;
                const float4 cc = C[c];
                const float bxh = C[c + 1].x, byh = C[c + CW].y, bzh = CN[c].z;
                const float pc = Pc[o];
                float v = cc.w * pc;
                v = fmaf(cc.x, pc - Pc[o - 1], v);
                v = fmaf(bxh, pc - Pc[o + 1], v);
                v = fmaf(cc.y, pc - Pc[o - SW], v);
                v = fmaf(byh, pc - Pc[o + SW], v);
                v = fmaf(cc.z, pc - PM[o], v);
                v = fmaf(bzh, pc - PP[o], v);
                q[og + 32 * k + sxy * z] = v;
                acc.add_prod(pc, v);
            }
        }
        __syncthreads();
    };
    const int zs = z0 - 1, zend = z1;  // p over zs .. zend, q over z0 .. z1-1
    fetch(zs, 0, 0);
    cp_commit();
    for (int zA = zs;;) {
        step(std::integral_constant<int, 0>{}, zA);
        if (++zA > zend) break;
        step(std::integral_constant<int, 1>{}, zA);
        if (++zA > zend) break;
        step(std::integral_constant<int, 2>{}, zA);
        if (++zA > zend) break;
        step(std::integral_constant<int, 3>{}, zA);
        if (++zA > zend) break;
    }
    cp_wait0();
    double v1[1] = {acc.total()};
    block_sum<1>(v1, sh);
    if (store_partials_is_last<1>(v1, partials, nblocks, &sc->ticket[10])) {
        double tot[1];
        finish_partials<1>(tot, partials, nblocks, sh, &sc->ticket[10]);
        if (t == 0) {
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
            sc->first = 0;
            sc->pidx = pidx_new;
        }
    }
}

// ------------------------------------------------------- smoother half-step
// Fine level: rhs = sigma * r (FP32), correction z (FP32), coefficients in the
// level precision.  ZERO: first half-step from zero (no vector staging).  The
// division uses the fast reciprocal: each cell's factor is a fixed number, so
// the sweep is still a fixed linear map and the V-cycle stays symmetric.
template <int CK, bool ZERO, bool OUT>
__global__ void __launch_bounds__(TILE_THREADS) k_smooth_staged(Grid3 g, const void* __restrict__ coef_v,
                                                                const float* __restrict__ r, float* e, float* out,
                                                                int color, const Scalars* sc) {
    if (sc->converged) return;
    using CT = typename CoefStore<CK>::T;
    const CT* coef = reinterpret_cast<const CT*>(coef_v);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto& R = *reinterpret_cast<Ring<CK>*>(smem_raw);
    const float sigma = sc->sigma;
    const int x0 = blockIdx.x * PX, y0 = blockIdx.y * TY;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x = x0 + 2 * tx, y = y0 + ty;
    const int z0 = blockIdx.z * g.zper, z1 = min(g.nz, z0 + g.zper);
    const bool inside = x < g.nx && y < g.ny;
    const Fetcher<CK> F(g, x0, y0);
    prologue<!ZERO, true>(F, R, z0, z1, e, coef, r);
    for (int z = z0; z < z1; z++) {
        advance<!ZERO, true>(F, R, z, z0, z1, e, coef, r);
        if (inside) {
            const int s = slot_of<CK>(z, z0), sp = slot_of<CK>(z + 1, z0);
            const int k = (color - (y + z)) & 1;  // the pair member of this colour
            const int cx = 2 * tx + k, ex = cx + 2;
            const float4 cc = unpack<CK>(R.c[s][ty][cx]);
            const float bxh = unpack<CK>(R.c[s][ty][cx + 1]).x;
            const float byh = unpack<CK>(R.c[s][ty + 1][cx]).y;
            const float bzh = unpack<CK>(R.c[sp][ty][cx]).z;
            const float d = ((cc.x + bxh) + (cc.y + byh)) + ((cc.z + bzh) + cc.w);
            float val = 0.f;
            if (d > 0.f) {
                float acc = sigma * R.r[s][ty][cx];
                if (!ZERO) {
                    const int sm = slot_of<CK>(z - 1, z0);
                    const float* er = &R.e[s][ty + 1][0];
                    acc = fmaf(cc.x, er[ex - 1], acc);
                    acc = fmaf(bxh, er[ex + 1], acc);
                    acc = fmaf(cc.y, R.e[s][ty][ex], acc);
                    acc = fmaf(byh, R.e[s][ty + 2][ex], acc);
                    acc = fmaf(cc.z, R.e[sm][ty + 1][ex], acc);
                    acc = fmaf(bzh, R.e[sp][ty + 1][ex], acc);
                }
                val = __fdividef(acc, d);
            }
            const long long i0 = x + (long long)g.nx * (y + (long long)g.ny * z);
            if (ZERO) {
                // both members written: the other colour starts at zero
                *reinterpret_cast<float2*>(e + i0) = k ? make_float2(0.f, val) : make_float2(val, 0.f);
            } else if (OUT) {
                out[i0 + k] = val;
            } else {
                e[i0 + k] = val;
            }
        }
        __syncthreads();
    }
    cp_wait0();
}

// -------------------------------------------------- residual + restriction
// rc[Q] = 1/4 sum over the 2x2x2 children of (sigma r - A z): the x pair is a
// thread's own two cells, the z pair two consecutive planes, the y pair goes
// through shared memory.  Requires an even z run per block.
template <int CK, class VTc>
__global__ void __launch_bounds__(TILE_THREADS) k_restrict_staged(Grid3 g, Grid3 gc, const void* __restrict__ coef_v,
                                                                  const float* __restrict__ r,
                                                                  const float* __restrict__ e, VTc* __restrict__ rc,
                                                                  const Scalars* sc) {
    if (sc->converged) return;
    using CT = typename CoefStore<CK>::T;
    const CT* coef = reinterpret_cast<const CT*>(coef_v);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto& R = *reinterpret_cast<Ring<CK>*>(smem_raw);
    __shared__ float ypart[TY][TX];
    const float sigma = sc->sigma;
    const int x0 = blockIdx.x * PX, y0 = blockIdx.y * TY;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x = x0 + 2 * tx, y = y0 + ty;
    const int z0 = blockIdx.z * g.zper, z1 = min(g.nz, z0 + g.zper);
    const bool inside = x < g.nx && y < g.ny;
    const Fetcher<CK> F(g, x0, y0);
    prologue<true, true>(F, R, z0, z1, e, coef, r);
    float part = 0.f;
    for (int z = z0; z < z1; z++) {
        advance<true, true>(F, R, z, z0, z1, e, coef, r);
        if (inside) {
            const int s = slot_of<CK>(z, z0), sm = slot_of<CK>(z - 1, z0), sp = slot_of<CK>(z + 1, z0);
            const float* er = &R.e[s][ty + 1][0];
#pragma unroll
            for (int k = 0; k < 2; k++) {
                const int cx = 2 * tx + k, ex = cx + 2;
                const float4 cc = unpack<CK>(R.c[s][ty][cx]);
                const float bxh = unpack<CK>(R.c[s][ty][cx + 1]).x;
                const float byh = unpack<CK>(R.c[s][ty + 1][cx]).y;
                const float bzh = unpack<CK>(R.c[sp][ty][cx]).z;
                const float d = ((cc.x + bxh) + (cc.y + byh)) + ((cc.z + bzh) + cc.w);
                float nsum = 0.f;
                nsum = fmaf(cc.x, er[ex - 1], nsum);
                nsum = fmaf(bxh, er[ex + 1], nsum);
                nsum = fmaf(cc.y, R.e[s][ty][ex], nsum);
                nsum = fmaf(byh, R.e[s][ty + 2][ex], nsum);
                nsum = fmaf(cc.z, R.e[sm][ty + 1][ex], nsum);
                nsum = fmaf(bzh, R.e[sp][ty + 1][ex], nsum);
                part += sigma * R.r[s][ty][cx] - (d * er[ex] - nsum);
            }
        }
        const bool last_of_pair = ((z - z0) & 1) || z + 1 == z1;
        if (last_of_pair) {
            ypart[ty][tx] = part;
            __syncthreads();
            if (inside && !(ty & 1)) {
                const float tot = part + ypart[ty + 1][tx];
                rc[(x >> 1) + (long long)gc.nx * ((y >> 1) + (long long)gc.ny * (z >> 1))] = from_f<VTc>(0.25f * tot);
            }
            part = 0.f;
        }
        __syncthreads();
    }
    cp_wait0();
}

// ------------------------------------------------------------ launchers
// Blocks per SM of each staged kernel (from the occupancy calculator) and the
// SM count: the z split is chosen so that the grid fills whole waves.
namespace {
int g_sms = 0;
int g_occ[8] = {0, 0, 0, 0, 0, 0, 0, 0};
enum { OCC_SPMV = 0, OCC_SMOOTH_F32, OCC_SMOOTH_LO, OCC_RESTRICT_F32, OCC_RESTRICT_LO, OCC_SEARCH };
}  // namespace

static Launch pair_launch(const Launch& L, int occ_kind) {
    Launch P = L;
    const int gx = (L.g.nx + PX - 1) / PX, gy = (L.g.ny + TY - 1) / TY, nz = L.g.nz;
    const int tiles = gx * gy;
    const int cap = (g_sms > 0 ? g_sms : 152) * (g_occ[occ_kind] > 0 ? g_occ[occ_kind] : 2);
    // candidate even z runs of at least 8 planes (or the whole column):
    // pick the one whose grid wastes the least of its last wave
    int best_zper = nz, best_zc = 1;
    double best = -1.0;
    for (int zc = 1; zc <= nz; zc++) {
        int zper = (nz + zc - 1) / zc;
        if ((zper & 1) && zper < nz) zper++;
        if (zper < 8 && zc > 1) break;
        const int zcr = (nz + zper - 1) / zper;
        const long long blocks = (long long)tiles * zcr;
        if (blocks > MAX_REDUCE_BLOCKS) break;
        const double waves = (double)blocks / cap;
        // fullness of the last wave times the share of fetched planes that
        // are computed (each run also fetches the planes just below and above)
        const double score = waves / std::ceil(waves) * ((double)zper / (zper + 2));
        if (score > best) {
            best = score;
            best_zper = zper;
            best_zc = zcr;
        }
    }
    P.grid = dim3(gx, gy, best_zc);
    P.g.zper = best_zper;
    P.nblocks = tiles * best_zc;
    return P;
}
bool staged_supported(const Grid3& g) { return (g.nx % 2) == 0; }

void launch_spmv_staged(const Launch& L, const Fields& F, cudaStream_t s) {
    const Launch P = pair_launch(L, OCC_SPMV);
    k_spmv_staged<<<P.grid, P.block, sizeof(Ring<0>), s>>>(P.g, F.coef, F.p, F.q, F.sc, F.partials, P.nblocks);
}

void launch_search_spmv(const Launch& L, const float4* coef, const float* z, const float* p_old, float* p_new,
                        float* x, float* q, Scalars* sc, double* partials, int pidx_new, cudaStream_t s) {
    const Launch P = pair_launch(L, OCC_SEARCH);
    k_search_spmv<<<P.grid, P.block, sizeof(SearchRing), s>>>(P.g, coef, z, p_old, p_new, x, q, sc, partials,
                                                              P.nblocks, pidx_new);
}

template <int CK>
static void smooth_staged_impl(const Launch& L, const void* coef, const float* r, float* e, float* tmp, int color,
                               bool zero, bool out_of_place, const Scalars* sc, cudaStream_t s) {
    const Launch P = pair_launch(L, CK == 0 ? OCC_SMOOTH_F32 : OCC_SMOOTH_LO);
    const size_t sm = sizeof(Ring<CK>);
    if (zero) k_smooth_staged<CK, true, false><<<P.grid, P.block, sm, s>>>(P.g, coef, r, e, e, color, sc);
    else if (!out_of_place) k_smooth_staged<CK, false, false><<<P.grid, P.block, sm, s>>>(P.g, coef, r, e, e, color, sc);
    else k_smooth_staged<CK, false, true><<<P.grid, P.block, sm, s>>>(P.g, coef, r, e, tmp, color, sc);
}
void launch_smooth_staged(int ck, const Launch& L, const void* coef, const float* r, float* e, float* tmp, int color,
                          bool zero, bool out_of_place, const Scalars* sc, cudaStream_t s) {
    if (ck == 1) smooth_staged_impl<1>(L, coef, r, e, tmp, color, zero, out_of_place, sc, s);
    else if (ck == 2) smooth_staged_impl<2>(L, coef, r, e, tmp, color, zero, out_of_place, sc, s);
    else smooth_staged_impl<0>(L, coef, r, e, tmp, color, zero, out_of_place, sc, s);
}

template <int CK, class VTc>
static void restrict_staged_impl(const Launch& L, const Grid3& gc, const void* coef, const float* r, const float* e,
                                 void* rc, const Scalars* sc, cudaStream_t s) {
    const Launch P = pair_launch(L, CK == 0 ? OCC_RESTRICT_F32 : OCC_RESTRICT_LO);
    k_restrict_staged<CK, VTc><<<P.grid, P.block, sizeof(Ring<CK>), s>>>(P.g, gc, coef, r, e, (VTc*)rc, sc);
}
void launch_restrict_staged(int ck, const Launch& L, const Grid3& gc, const void* coef, const float* r, const float* e,
                            void* rc, const Scalars* sc, cudaStream_t s) {
    if (ck == 1) restrict_staged_impl<1, __half>(L, gc, coef, r, e, rc, sc, s);
    else if (ck == 2) restrict_staged_impl<2, __nv_bfloat16>(L, gc, coef, r, e, rc, sc, s);
    else restrict_staged_impl<0, float>(L, gc, coef, r, e, rc, sc, s);
}

cudaError_t staged_prepare_attributes() {
    cudaError_t e = cudaSuccess;
    auto set = [&](const void* fn, size_t bytes) {
        if (e == cudaSuccess) e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    };
    set((const void*)k_spmv_staged, sizeof(Ring<0>));
    set((const void*)k_search_spmv, sizeof(SearchRing));
    set((const void*)k_smooth_staged<0, true, false>, sizeof(Ring<0>));
    set((const void*)k_smooth_staged<0, false, false>, sizeof(Ring<0>));
    set((const void*)k_smooth_staged<0, false, true>, sizeof(Ring<0>));
    set((const void*)k_smooth_staged<1, true, false>, sizeof(Ring<1>));
    set((const void*)k_smooth_staged<1, false, false>, sizeof(Ring<1>));
    set((const void*)k_smooth_staged<1, false, true>, sizeof(Ring<1>));
    set((const void*)k_smooth_staged<2, true, false>, sizeof(Ring<2>));
    set((const void*)k_smooth_staged<2, false, false>, sizeof(Ring<2>));
    set((const void*)k_smooth_staged<2, false, true>, sizeof(Ring<2>));
    set((const void*)k_restrict_staged<0, float>, sizeof(Ring<0>));
    set((const void*)k_restrict_staged<1, __half>, sizeof(Ring<1>));
    set((const void*)k_restrict_staged<2, __nv_bfloat16>, sizeof(Ring<2>));
    if (e != cudaSuccess) return e;
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
    auto occ = [&](int kind, const void* fn, size_t bytes) {
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_occ[kind], fn, TILE_THREADS, bytes);
    };
    occ(OCC_SPMV, (const void*)k_spmv_staged, sizeof(Ring<0>));
    occ(OCC_SEARCH, (const void*)k_search_spmv, sizeof(SearchRing));
    occ(OCC_SMOOTH_F32, (const void*)k_smooth_staged<0, false, false>, sizeof(Ring<0>));
    occ(OCC_SMOOTH_LO, (const void*)k_smooth_staged<1, false, false>, sizeof(Ring<1>));
    occ(OCC_RESTRICT_F32, (const void*)k_restrict_staged<0, float>, sizeof(Ring<0>));
    occ(OCC_RESTRICT_LO, (const void*)k_restrict_staged<1, __half>, sizeof(Ring<1>));
    return e;
}

}  // namespace mhdproj
