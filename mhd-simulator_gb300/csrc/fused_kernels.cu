// fused_kernels.cu -- the multigrid V-cycle's per-level work in two passes
// over HBM instead of six.
//
// Pre-smoothing pass (k_presmooth_restrict), per level:
//   [fine level, inside CG] r <- r - alpha q       (the CG residual update)
//   red half-step from a zero correction            e_red   = sigma r / d
//   black half-step                                 e_black = (sigma r + sum beta e_red) / d
//   residual and restriction                        rc      = 1/4 P^T (sigma r - A e)
// Post-smoothing pass (k_prolong_postsmooth), per level:
//   prolongation                                    e <- e + w P ec
//   black half-step, then red half-step             z       = the smoothed correction
//   [fine level] r . z for the CG step length.
// Both march a 64 x 16 (x, y) tile along z.  The stages of one pass run as a
// pipeline over planes: the pre-smoothing pass forms the residual and the red
// values of plane z, the black values of plane z-1 and the restricted
// residual of plane z-2 in the same step, so every input plane is read from
// HBM once.  A stage needs its neighbours' results, so each stage runs on a
// region one cell wider than the next: the red values cover the tile with a
// 2-cell halo, the black values a 1-cell halo, the residual the tile itself.
// Halo cells are recomputed by both neighbouring tiles from the same inputs
// in the same order, so the values agree bit for bit.
//
// Work is split in quads, four consecutive cells x0-4+4q .. x0-1+4q of a
// row.  x0-4 is even, so in a quad the cells of one colour are the two cells
// of one x parity.  Shared-memory planes are [rows][2][36]: each staged row
// (x0-4 .. x0+67) holds its even-x cells, then its odd-x cells, so a quad's
// cells of one colour are two adjacent floats and a warp's accesses are
// contiguous.  The smoother records are staged one plane ahead with
// zero-filling 16-byte cp.async (the records in HBM use the same split along
// whole grid rows, so a staged half row is one contiguous run); the red
// stage's vector inputs go to registers, loaded once the stage has consumed
// the previous plane's.  Three barriers per plane.
//
// The smoother reads per-cell records (beta_x, beta_y, beta_z of the low
// faces, diagonal) prepared once per coefficient set, the diagonal rounded
// up to the record precision: the level operator stays diagonally dominant,
// so the V-cycle stays a fixed symmetric positive definite operator.
// Requirements: nx a multiple of 4 and even extents on periodic axes.
#include <algorithm>
#include <cmath>
#include <type_traits>

#include "kernels.h"
#include "fused_common.cuh"

namespace mhdproj {

namespace {
using namespace staged;
using namespace fused;

// Tile rows: 16 with 8-byte (FP16/BF16) records, 8 with 16-byte (FP32)
// records, so that three blocks fit the shared memory of an SM.
template <int FTY_>
struct Geo {
    static constexpr int FTY = FTY_;               // one thread row per tile row
    static constexpr int FT = QX * FTY;            // threads per block
    static constexpr int RH = FTY + 4;             // vector rows:  y0-2 .. y0+FTY+1
    static constexpr int CH = FTY + 5;             // record rows:  y0-2 .. y0+FTY+2
    static constexpr int NRED = RH * NQ;           // red-stage quads (rows y0-2 .. y0+FTY+1)
    static constexpr int NBLK = (FTY + 2) * NQ;    // black-stage quads (rows y0-1 .. y0+FTY)
    static_assert(NRED <= 2 * FT && NBLK <= 2 * FT, "two tasks per thread");
};
template <int CK>
using GeoOf = Geo<CK == 0 ? 8 : 16>;

// A thread's share of one plane's record copies, resolved once per block:
// NCT 16-byte copies of the record rows (21 rows x 2 half rows x 36
// 8-byte records, or 13 rows x 2 x 36 16-byte records).  A copy of two 8-byte
// records covers cells x and x+2 of a quad, so both exist or neither does
// (nx is a multiple of 4).
template <int CK>
struct RecordFetch {
    using CT = typename CoefStore<CK>::T;
    using G = GeoOf<CK>;
    static constexpr int FT = G::FT;
    static constexpr int RPC = (CK == 0) ? 1 : 2;  // records per 16-byte copy
    static constexpr int PER = HW / RPC;           // copies per half row
    static constexpr int NCTOT = G::CH * 2 * PER;
    static constexpr int NCT = (NCTOT + FT - 1) / FT;
    int coff[NCT];
    short cdst[NCT];
    bool cok[NCT];
    long long sxy;
    int nz;
    bool pz;

    __device__ __forceinline__ RecordFetch(const Grid3& g, int x0, int y0, int t) {
        sxy = (long long)g.nx * g.ny;
        nz = g.nz;
        pz = (g.periodic & 4) != 0;
        const bool px = g.periodic & 1, py = g.periodic & 2;
#pragma unroll
        for (int j = 0; j < NCT; j++) {
            const int k = t + j * FT;
            cdst[j] = -1;
            cok[j] = false;
            coff[j] = 0;
            if (k < NCTOT) {
                const int row = k / (2 * PER), rem = k - row * 2 * PER;
                const int h = rem / PER, ci = rem - h * PER;
                bool okx, oky;
                const int sx = axis_src(x0 - XO + 2 * RPC * ci, g.nx, px, &okx);  // even cell of the copy
                const int sy = axis_src(y0 - 2 + row, g.ny, py, &oky);
                cok[j] = okx && oky;
                coff[j] = cok[j] ? g.nx * sy + h * (g.nx >> 1) + (sx >> 1) : 0;
                cdst[j] = (short)(row * RW + h * HW + RPC * ci);
            }
        }
    }
    __device__ __forceinline__ long long plane(int zz, bool* okz) const {
        const int sz = axis_src(zz, nz, pz, okz);
        return (long long)sz * sxy;
    }
    __device__ __forceinline__ void recs(CT* dst, const CT* src, long long pl, bool okz) const {
#pragma unroll
        for (int j = 0; j < NCT; j++)
            if (cdst[j] >= 0) {
                const bool ok = cok[j] && okz;
                cp_async16(dst + cdst[j], src + (ok ? pl + coff[j] : 0), ok);
            }
    }
};

// A thread's quad tasks of the red / prolongation (2-halo rows, quads 0..17)
// and black (1-halo rows) stages, resolved once per block: the split-plane
// offset of the quad's even half (the odd half is HW further), the row's y,
// the quad's in-plane offset in the grid (wrapped on periodic axes) and
// whether it exists, and for quads on the tile the unwrapped in-plane offset
// (-1 otherwise).  Cells outside the regions (quads 0 and 17 reach two cells
// beyond the 2-halo) are computed like the others and never read.
template <class G>
struct QuadTasks {
    static constexpr int FT = G::FT, FTY = G::FTY, NRED = G::NRED, NBLK = G::NBLK;
    int roff[2], ry[2], rown[2], goff[2];
    bool gok[2];
    int boff[2], by[2];
    __device__ __forceinline__ QuadTasks(const Grid3& g, int x0, int y0, int t) {
        const bool px = g.periodic & 1, py = g.periodic & 2;
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int k = t + u * FT;
            roff[u] = -1;
            ry[u] = 0;
            rown[u] = -1;
            goff[u] = 0;
            gok[u] = false;
            if (k < NRED) {
                const int row = k / NQ, q = k - row * NQ;
                roff[u] = row * RW + 2 * q;
                const int gx = x0 - XO + 4 * q, gy = y0 - 2 + row;
                ry[u] = gy;
                if (row >= 2 && row < FTY + 2 && q >= 1 && q <= QX && gx < g.nx && gy < g.ny) rown[u] = gx + g.nx * gy;
                bool okx, oky;
                const int sx = axis_src(gx, g.nx, px, &okx);
                const int sy = axis_src(gy, g.ny, py, &oky);
                gok[u] = okx && oky;
                goff[u] = gok[u] ? sx + g.nx * sy : 0;
            }
            boff[u] = -1;
            by[u] = 0;
            if (k < NBLK) {
                const int rb = k / NQ, q = k - rb * NQ, row = rb + 1;
                boff[u] = row * RW + 2 * q;
                by[u] = y0 - 2 + row;
            }
        }
    }
};
// Plane rings in shared memory.  A step handles planes zA (red /
// prolongation stage), zA-1 (black stage) and zA-2 (tile stage) and stages
// the records of plane zA+1 for the next step; rings of 4 planes, so the z
// loop is unrolled four times and every slot is a compile-time offset.  In
// the correction ring the black cells of the newest plane hold their
// right-hand side sigma r until the black stage replaces it by their value.
template <int CK>
struct PreRing {
    using CT = typename CoefStore<CK>::T;
    using G = GeoOf<CK>;
    CT c[4][G::CH][RW];              // records, planes zA-2 .. zA+1
    float er[4][G::RH][RW];          // correction, planes zA-3 .. zA
    float2 ypart[G::FTY][QX];
};
template <int CK>
struct PostRing {
    using CT = typename CoefStore<CK>::T;
    using G = GeoOf<CK>;
    CT c[4][G::CH][RW];              // records, planes zA-2 .. zA+1
    float ep[4][G::RH][RW];          // prolonged / smoothed correction, planes zA-3 .. zA
};
constexpr int FUSED_MIN_BLOCKS = 3;
}  // namespace

// ------------------------------------------------------ pre-smoothing pass
// Level residual rin (VT) -> correction e (VT, own cells) and the coarse
// residual rc.  UPDATE (finest level inside CG): the residual is first
// updated, r_out = rin - alpha q, written for the tile's cells, and ||r_out||^2
// decides convergence.  FINE: the right-hand side is sigma * r.
// After the two half-steps the residual of a black cell is zero (its update
// solves its own equation) and that of a red cell is sum beta * e over its
// black neighbours (its red value solved the equation with them at zero), so
// the restriction sums those neighbour terms over the red cells.
// rin and q must not alias r_out (other tiles read them as halo).
template <int CK, class VT, class VTc, bool UPDATE, bool FINE>
__global__ void __launch_bounds__(GeoOf<CK>::FT, FUSED_MIN_BLOCKS)
    k_presmooth_restrict(Grid3 g, Grid3 gc, const void* __restrict__ sm_v, const VT* __restrict__ rin,
                         const float* __restrict__ q, float* __restrict__ r_out, VT* __restrict__ e,
                         VTc* __restrict__ rc, Scalars* sc, double* partials, int nblocks) {
    if (sc->converged) return;
    using CT = typename CoefStore<CK>::T;
    using G = GeoOf<CK>;
    constexpr int FTY = G::FTY, FT = G::FT;
    using R4 = typename Raw4<VT>::T;
    const CT* sm = reinterpret_cast<const CT*>(sm_v);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto& S = *reinterpret_cast<PreRing<CK>*>(smem_raw);
    __shared__ double sh[FT / 32];
    const float sigma = FINE ? sc->sigma : 1.0f;
    const float alpha = UPDATE ? sc->alpha_f : 0.0f;
    const int x0 = blockIdx.x * PX, y0 = blockIdx.y * FTY;
    const int tx = threadIdx.x, ty = threadIdx.y, t = tx + QX * ty;
    const int z0 = blockIdx.z * g.zper, z1 = min(g.nz, z0 + g.zper);
    const RecordFetch<CK> F(g, x0, y0, t);
    const QuadTasks<G> T(g, x0, y0, t);
    const long long sxy = (long long)g.nx * g.ny;
    // ||r||^2 only steers the stop test and sigma: a per-thread FP32 sum,
    // FP64 across threads and blocks
    float rr_thread = 0.f;
    float2 part = make_float2(0.f, 0.f);  // restriction sums of the own quad's two parents
    int rc_z = -1;  // coarse plane whose restriction awaits the row pair sum
    const int ox = x0 + 4 * tx, oy = y0 + ty;  // the thread's own quad
    const bool own_inside = ox < g.nx && oy < g.ny;
    const int oo = (ty + 2) * RW + 2 * (tx + 1);  // split offset of its even half
    const long long og = ox + (long long)g.nx * oy;
    R4 rv[2];
    float4 qv[2];
    auto stage = [&](int zz, int c4) {
        bool okz;
        const long long pl = F.plane(zz, &okz);
        F.recs(&S.c[c4][0][0], sm, pl, okz);
        cp_commit();
    };
    auto load = [&](int zz) {  // the red tasks' residual (and q) of plane zz
        bool okz;
        const long long pl = F.plane(zz, &okz);
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const bool ok = T.gok[u] && okz;
            rv[u] = ldg_quad<VT>(rin + pl + T.goff[u], ok);
            if (UPDATE) qv[u] = ok ? __ldg(reinterpret_cast<const float4*>(q + pl + T.goff[u])) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    };
    auto flush_rc = [&]() {
        if (rc_z >= 0 && own_inside && !(ty & 1)) {
            const float2 a = S.ypart[ty][tx], b = S.ypart[ty + 1][tx];
            st2<VTc>(rc + (ox >> 1) + (long long)gc.nx * ((oy >> 1) + (long long)gc.ny * rc_z),
                     make_float2(0.25f * (a.x + b.x), 0.25f * (a.y + b.y)));
        }
        rc_z = -1;
    };
    auto step = [&](auto ph, int zA) {
        constexpr int P = decltype(ph)::value;
        cp_wait<0>();
        __syncthreads();
        stage(zA + 1, (P + 1) & 3);
        flush_rc();
        // ---- red stage: plane zA over the 2-halo rows
        {
            const CT* C = &S.c[P][0][0];
            float* ER = &S.er[P][0][0];
            const bool zin = zA >= z0 && zA < z1;
            float* rplane = UPDATE ? r_out + sxy * zA : nullptr;
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const int o = T.roff[u];
                if (o < 0) break;
                float4 rn = cvt4r<VT>(rv[u]);
                if (UPDATE)
                    rn = make_float4(fmaf(-alpha, qv[u].x, rn.x), fmaf(-alpha, qv[u].y, rn.y),
                                     fmaf(-alpha, qv[u].z, rn.z), fmaf(-alpha, qv[u].w, rn.w));
                const int p = red_half(T.ry[u], zA);
                float4 d0, d1;
                rec2<CK>(C + o + p * HW, &d0, &d1);
                const float2 rr = p ? make_float2(rn.y, rn.w) : make_float2(rn.x, rn.z);  // red cells
                const float2 rb = p ? make_float2(rn.x, rn.z) : make_float2(rn.y, rn.w);  // black cells
                const float2 ev = divide2(make_float2(sigma * rr.x, sigma * rr.y), make_float2(d0.w, d1.w));
                *reinterpret_cast<float2*>(ER + o + p * HW) = ev;
                *reinterpret_cast<float2*>(ER + o + (1 - p) * HW) = make_float2(sigma * rb.x, sigma * rb.y);
                if (UPDATE && zin && T.rown[u] >= 0) {
                    *reinterpret_cast<float4*>(rplane + T.rown[u]) = rn;
                    rr_thread = fmaf(rn.x, rn.x, fmaf(rn.y, rn.y, fmaf(rn.z, rn.z, fmaf(rn.w, rn.w, rr_thread))));
                }
            }
        }
        load(zA + 1);
        __syncthreads();
        // ---- black stage: plane zA-1 over the 1-halo rows, in place
        const int zB = zA - 1;
        if (zB >= z0 - 1) {
            const CT* C = &S.c[(P + 3) & 3][0][0];
            const CT* CN = &S.c[P][0][0];
            float* E = &S.er[(P + 3) & 3][0][0];
            const float* EM = &S.er[(P + 2) & 3][0][0];
            const float* EP = &S.er[P][0][0];
#pragma unroll
            for (int u = 0; u < 2; u++) {
                if (T.boff[u] < 0) break;
                const int h = 1 - red_half(T.by[u], zB);
                const int o = T.boff[u] + h * HW;
                float2 d;
                const float2 s = gs_sum2<CK>(C, CN, E, EM, EP, o, h, *reinterpret_cast<const float2*>(E + o), &d);
                *reinterpret_cast<float2*>(E + o) = divide2(s, d);
            }
        }
        __syncthreads();
        // ---- correction out and restriction: plane zA-2 over the tile
        const int zC = zA - 2;
        if (zC >= z0 && zC < z1) {
            const CT* C = &S.c[(P + 2) & 3][0][0];
            const CT* CN = &S.c[(P + 3) & 3][0][0];
            const float* E = &S.er[(P + 2) & 3][0][0];
            const float* EM = &S.er[(P + 1) & 3][0][0];
            const float* EP = &S.er[(P + 3) & 3][0][0];
            const int p = red_half(oy, zC);  // red half of the own quad
            float2 d;
            const float2 s = gs_sum2<CK>(C, CN, E, EM, EP, oo + p * HW, p, make_float2(0.f, 0.f), &d);
            part.x += s.x;
            part.y += s.y;
            if (own_inside) {
                const float2 ev = *reinterpret_cast<const float2*>(E + oo);
                const float2 od = *reinterpret_cast<const float2*>(E + oo + HW);
                st4<VT>(e + (og + sxy * zC), make_float4(ev.x, od.x, ev.y, od.y));
            }
            if (((zC - z0) & 1) || zC + 1 == z1) {
                // the row pair sum is formed after the next barrier
                S.ypart[ty][tx] = part;
                rc_z = zC >> 1;
                part = make_float2(0.f, 0.f);
            }
        }
    };
    const int zs = z0 - 2, zend = z1 + 1;  // red stage over zs .. zend
    stage(zs, 0);
    load(zs);
    for (int zA = zs;;) {
        step(Phase<0>{}, zA);
        if (++zA > zend) break;
        step(Phase<1>{}, zA);
        if (++zA > zend) break;
        step(Phase<2>{}, zA);
        if (++zA > zend) break;
        step(Phase<3>{}, zA);
        if (++zA > zend) break;
    }
    cp_wait<0>();
    __syncthreads();
    flush_rc();
    if (UPDATE) {
        double v1[1] = {(double)rr_thread};
        block_sum<1>(v1, sh);
        if (store_partials_is_last<1>(v1, partials, nblocks, &sc->ticket[8])) {
            double tot[1];
            finish_partials<1>(tot, partials, nblocks, sh, &sc->ticket[8]);
            if (t == 0) {
                const double rr = tot[0];
                sc->rr = rr;
                sc->iterations += 1;
                sc->total_iterations += 1;
                if (!isfinite(rr)) {
                    sc->nonfinite = 1;
                    sc->converged = 1;
                } else if (rr <= sc->rr_target || sc->total_iterations >= sc->max_total) {
                    sc->converged = 1;
                }
            }
        }
    }
}

// ----------------------------------------------------- post-smoothing pass
// e (pre-smoothed, VT) + w * P ec -> black, red half-steps -> out (VT).  DOT
// (finest level): r . out / sigma gives rz and beta; the next V-cycle's sigma
// is then taken from ||r||^2.  The black half-step does not read a black
// cell's own prolonged value, so the prolongation stage leaves sigma r there.
template <int CK, class VT, class VTc, bool DOT, bool FINE>
__global__ void __launch_bounds__(GeoOf<CK>::FT, FUSED_MIN_BLOCKS)
    k_prolong_postsmooth(Grid3 g, Grid3 gc, const void* __restrict__ sm_v, const VT* __restrict__ e,
                         const VTc* __restrict__ ec, const VT* __restrict__ r, VT* __restrict__ out,
                         const VT* __restrict__ accum, float w, Scalars* sc, double* partials, int nblocks,
                         long long n_active) {
    if (sc->converged) return;
    using CT = typename CoefStore<CK>::T;
    using G = GeoOf<CK>;
    constexpr int FTY = G::FTY, FT = G::FT;
    using R4 = typename Raw4<VT>::T;
    using C2 = typename Raw2<VTc>::T;
    const CT* sm = reinterpret_cast<const CT*>(sm_v);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto& S = *reinterpret_cast<PostRing<CK>*>(smem_raw);
    __shared__ double sh[FT / 32];
    const float sigma = FINE ? sc->sigma : 1.0f;
    const float is = FINE ? sc->inv_sigma : 1.0f;
    const int x0 = blockIdx.x * PX, y0 = blockIdx.y * FTY;
    const int tx = threadIdx.x, ty = threadIdx.y, t = tx + QX * ty;
    const int z0 = blockIdx.z * g.zper, z1 = min(g.nz, z0 + g.zper);
    const RecordFetch<CK> F(g, x0, y0, t);
    const QuadTasks<G> T(g, x0, y0, t);
    const long long sxy = (long long)g.nx * g.ny;
    // coarse parents of the red-stage quads: in-plane offsets of the pair
    int pofs[2];
    {
        const bool px = g.periodic & 1, py = g.periodic & 2;
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int k = t + u * FT;
            pofs[u] = 0;
            if (k < G::NRED) {
                const int row = k / NQ, qq = k - row * NQ;
                bool okx, oky;
                const int sx = axis_src(x0 - XO + 4 * qq, g.nx, px, &okx);
                const int sy = axis_src(y0 - 2 + row, g.ny, py, &oky);
                pofs[u] = (okx && oky) ? (sx >> 1) + gc.nx * (sy >> 1) : 0;
            }
        }
    }
    const long long csxy = (long long)gc.nx * gc.ny;
    Acc acc;
    const int ox = x0 + 4 * tx, oy = y0 + ty;
    const bool own_inside = ox < g.nx && oy < g.ny;
    const int oo = (ty + 2) * RW + 2 * (tx + 1);
    const long long og = ox + (long long)g.nx * oy;
    // registers of the red-stage quads of the next plane: the pre-smoothed
    // correction, the right-hand side (for the black cells) and the coarse
    // parents; and the own quad's right-hand side of the tile plane
    R4 eov[2], rqv[2];
    C2 pcv[2];
    R4 rov, ron;
    auto stage = [&](int zz, int c4) {
        bool okz;
        const long long pl = F.plane(zz, &okz);
        F.recs(&S.c[c4][0][0], sm, pl, okz);
        cp_commit();
    };
    auto load = [&](int zz) {
        bool okz;
        const int sz = axis_src(zz, g.nz, (g.periodic & 4) != 0, &okz);
        const long long pl = (long long)sz * sxy, cpl = (long long)(sz >> 1) * csxy;
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const bool ok = T.gok[u] && okz;
            eov[u] = ldg_quad<VT>(e + pl + T.goff[u], ok);
            rqv[u] = ldg_quad<VT>(r + pl + T.goff[u], ok);
            pcv[u] = ldg_pair<VTc>(ec + cpl + pofs[u], ok);
        }
        const int zt = zz - 2;  // the tile plane of the step that uses this plane's red stage
        ron = ldg_quad<VT>(r + og + sxy * zt, own_inside && zt >= z0 && zt < z1);
    };
    auto step = [&](auto ph, int zA) {
        constexpr int P = decltype(ph)::value;
        cp_wait<0>();
        __syncthreads();
        stage(zA + 1, (P + 1) & 3);
        rov = ron;
        // ---- prolongation: plane zA over the 2-halo rows
        {
            float* EP = &S.ep[P][0][0];
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const int o = T.roff[u];
                if (o < 0) break;
                const float4 ev = cvt4r<VT>(eov[u]);
                const float4 rq = cvt4r<VT>(rqv[u]);
                const float2 cv = cvt2(pcv[u]);
                const int p = red_half(T.ry[u], zA);
                const float2 er = p ? make_float2(ev.y, ev.w) : make_float2(ev.x, ev.z);
                const float2 rb = p ? make_float2(rq.x, rq.z) : make_float2(rq.y, rq.w);
                *reinterpret_cast<float2*>(EP + o + p * HW) = make_float2(fmaf(w, cv.x, er.x), fmaf(w, cv.y, er.y));
                *reinterpret_cast<float2*>(EP + o + (1 - p) * HW) = make_float2(sigma * rb.x, sigma * rb.y);
            }
        }
        load(zA + 1);
        __syncthreads();
        // ---- black half-step: plane zA-1 over the 1-halo rows, in place
        const int zB = zA - 1;
        if (zB >= z0 - 1) {
            const CT* C = &S.c[(P + 3) & 3][0][0];
            const CT* CN = &S.c[P][0][0];
            float* E = &S.ep[(P + 3) & 3][0][0];
            const float* EM = &S.ep[(P + 2) & 3][0][0];
            const float* EP = &S.ep[P][0][0];
#pragma unroll
            for (int u = 0; u < 2; u++) {
                if (T.boff[u] < 0) break;
                const int h = 1 - red_half(T.by[u], zB);
                const int o = T.boff[u] + h * HW;
                float2 d;
                const float2 s = gs_sum2<CK>(C, CN, E, EM, EP, o, h, *reinterpret_cast<const float2*>(E + o), &d);
                *reinterpret_cast<float2*>(E + o) = divide2(s, d);
            }
        }
        __syncthreads();
        // ---- red half-step: plane zA-2 over the tile, out = z
        const int zC = zA - 2;
        if (zC >= z0 && zC < z1) {
            const CT* C = &S.c[(P + 2) & 3][0][0];
            const CT* CN = &S.c[(P + 3) & 3][0][0];
            const float* E = &S.ep[(P + 2) & 3][0][0];
            const float* EM = &S.ep[(P + 1) & 3][0][0];
            const float* EP = &S.ep[(P + 3) & 3][0][0];
            const int p = red_half(oy, zC);
            const float4 rv = cvt4r<VT>(rov);
            const float2 rr = p ? make_float2(rv.y, rv.w) : make_float2(rv.x, rv.z);
            float2 d;
            const float2 s = gs_sum2<CK>(C, CN, E, EM, EP, oo + p * HW, p, make_float2(sigma * rr.x, sigma * rr.y), &d);
            const float2 zr = divide2(s, d);
            const float2 zb = *reinterpret_cast<const float2*>(E + oo + (1 - p) * HW);
            float4 zv = p ? make_float4(zb.x, zr.x, zb.y, zr.y) : make_float4(zr.x, zb.x, zr.y, zb.y);
            if (own_inside) {
                if (accum) {  // out = accum + z (second W-cycle visit)
                    const float4 a = cvt4r<VT>(*reinterpret_cast<const R4*>(accum + og + sxy * zC));
                    zv = make_float4(a.x + zv.x, a.y + zv.y, a.z + zv.z, a.w + zv.w);
                }
                st4<VT>(out + og + sxy * zC, zv);
                if (DOT) {
                    acc.add_prod(rv.x, zv.x * is);
                    acc.add_prod(rv.y, zv.y * is);
                    acc.add_prod(rv.z, zv.z * is);
                    acc.add_prod(rv.w, zv.w * is);
                }
            }
        }
    };
    const int zs = z0 - 2, zend = z1 + 1;
    stage(zs, 0);
    load(zs);
    for (int zA = zs;;) {
        step(Phase<0>{}, zA);
        if (++zA > zend) break;
        step(Phase<1>{}, zA);
        if (++zA > zend) break;
        step(Phase<2>{}, zA);
        if (++zA > zend) break;
        step(Phase<3>{}, zA);
        if (++zA > zend) break;
    }
    cp_wait<0>();
    if (DOT) {
        double v1[1] = {acc.total()};
        block_sum<1>(v1, sh);
        if (store_partials_is_last<1>(v1, partials, nblocks, &sc->ticket[9])) {
            double tot[1];
            finish_partials<1>(tot, partials, nblocks, sh, &sc->ticket[9]);
            if (t == 0) {
                const double rz = tot[0];
                if (!isfinite(rz)) {
                    sc->nonfinite = 1;
                    sc->converged = 1;
                } else if (!(rz > 0.0)) {
                    sc->breakdown = 1;
                    sc->converged = 1;
                } else if (sc->first) {
                    sc->rz = rz;
                    sc->beta = 0.0;
                    sc->beta_f = 0.0f;
                } else {
                    sc->beta = rz / sc->rz;
                    sc->beta_f = (float)sc->beta;
                    sc->rz = rz;
                }
                // z is in units of this V-cycle's sigma; the next V-cycle
                // scales by the RMS of the residual it will be given.
                sc->inv_sigma_z = sc->inv_sigma;
                set_sigma_from(sc, sc->rr, n_active);
            }
        }
    }
}

// --------------------------------------------------- smoother records
// (beta_x, beta_y, beta_z, diagonal) per cell from the level's coefficient
// records (beta_x, beta_y, beta_z, reaction); the diagonal is the FP32 sum of
// the record-precision values, rounded up to the record precision.  Stored
// with each grid row split into its even-x and odd-x halves (split_x).
template <int CK>
__global__ void __launch_bounds__(TILE_THREADS) k_smoother_records(Grid3 g, const void* __restrict__ coef_v,
                                                                   void* __restrict__ sm_v) {
    using CT = typename CoefStore<CK>::T;
    const CT* coef = reinterpret_cast<const CT*>(coef_v);
    CT* sm = reinterpret_cast<CT*>(sm_v);
    const int x = blockIdx.x * TX + threadIdx.x, y = blockIdx.y * TY + threadIdx.y;
    if (x >= g.nx || y >= g.ny) return;
    const int z0 = blockIdx.z * g.zper, z1 = min(g.nz, z0 + g.zper);
    const long long sy = g.nx, sz = (long long)g.nx * g.ny;
    for (int z = z0; z < z1; z++) {
        const long long i = x + sy * y + sz * z;
        const float4 c = unpack<CK>(coef[i]);
        const int xp = wrap_or_neg(x + 1, g.nx, g.periodic & 1);
        const int yp = wrap_or_neg(y + 1, g.ny, g.periodic & 2);
        const int zp = wrap_or_neg(z + 1, g.nz, g.periodic & 4);
        const float bxh = xp >= 0 ? unpack<CK>(coef[xp + sy * y + sz * z]).x : 0.f;
        const float byh = yp >= 0 ? unpack<CK>(coef[x + sy * yp + sz * z]).y : 0.f;
        const float bzh = zp >= 0 ? unpack<CK>(coef[x + sy * y + sz * zp]).z : 0.f;
        const float d = ((c.x + bxh) + (c.y + byh)) + ((c.z + bzh) + c.w);
        CT out;
        if (CK == 0) {
            reinterpret_cast<float4&>(out) = make_float4(c.x, c.y, c.z, d);
        } else {
            // the three betas are exact in the record precision already
            uint2 u = reinterpret_cast<const uint2&>(coef[i]);
            unsigned short dh;
            if (CK == 1) {
                const __half h = __float2half_ru(d);
                dh = *reinterpret_cast<const unsigned short*>(&h);
            } else {
                const __nv_bfloat16 h = __float2bfloat16_ru(d);
                dh = *reinterpret_cast<const unsigned short*>(&h);
            }
            u.y = (u.y & 0x0000ffffu) | ((unsigned)dh << 16);
            reinterpret_cast<uint2&>(out) = u;
        }
        sm[i + (split_x(x, g.nx) - x)] = out;
    }
}

// ------------------------------------------------------------ launchers
namespace {
int f_sms = 0;
int f_occ[12] = {};
enum { O_PRE_F32 = 0, O_PRE_LO, O_PRE_LO_UPD, O_PRE_F32_UPD, O_PRE_COARSE, O_POST_F32, O_POST_LO, O_POST_COARSE };

// Even z runs chosen so the grid fills whole waves of resident blocks; each
// run also computes two planes below and above it.  On levels too small to
// fill one wave the score favours the shortest runs (fewest steps per block).
Launch fused_launch(const Grid3& g0, int occ_kind, int fty) {
    Launch P;
    P.g = g0;
    P.block = dim3(QX, fty, 1);
    const int gx = (g0.nx + PX - 1) / PX, gy = (g0.ny + fty - 1) / fty, nz = g0.nz;
    const int tiles = gx * gy;
    const int cap = (f_sms > 0 ? f_sms : 152) * (f_occ[occ_kind] > 0 ? f_occ[occ_kind] : 1);
    int best_zper = nz + (nz & 1), best_zc = 1;
    double best = -1.0;
    for (int zc = 1; zc <= nz; zc++) {
        int zper = (nz + zc - 1) / zc;
        if (zper & 1) zper++;
        if (zper < 2 && zc > 1) break;
        const int zcr = (nz + zper - 1) / zper;
        const long long blocks = (long long)tiles * zcr;
        if (blocks > MAX_REDUCE_BLOCKS) break;
        const double waves = (double)blocks / cap;
        const double score = waves / std::ceil(waves) * ((double)zper / (zper + 4));
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
}  // namespace

bool fused_supported(const Grid3& g) {
    if (g.nx % 4) return false;
    for (int a = 0; a < 3; a++) {
        const int n = a == 0 ? g.nx : (a == 1 ? g.ny : g.nz);
        if ((g.periodic & (1 << a)) && (n & 1)) return false;
    }
    return true;
}

template <int CK, class VT, class VTc, bool UPDATE, bool FINE>
static void pre_impl(const Grid3& g, const Grid3& gc, const void* sm, const void* rin, const float* q, float* r_out,
                     void* e, void* rc, Scalars* sc, double* partials, int occ_kind, cudaStream_t s) {
    if (tma_pre(CK, FINE, UPDATE, g, gc, sm, rin, q, r_out, e, rc, sc, partials, s)) return;
    const Launch P = fused_launch(g, occ_kind, GeoOf<CK>::FTY);
    k_presmooth_restrict<CK, VT, VTc, UPDATE, FINE><<<P.grid, P.block, sizeof(PreRing<CK>), s>>>(
        P.g, gc, sm, (const VT*)rin, q, r_out, (VT*)e, (VTc*)rc, sc, partials, P.nblocks);
}
template <int CK, class VT, class VTc, bool DOT, bool FINE>
static void post_impl(const Grid3& g, const Grid3& gc, const void* sm, const void* e, const void* ec, const void* r,
                      void* out, const void* accum, float w, Scalars* sc, double* partials, long long n_active,
                      int occ_kind, cudaStream_t s) {
    if (tma_post(CK, FINE, g, gc, sm, e, ec, r, out, accum, w, sc, partials, n_active, s)) return;
    const Launch P = fused_launch(g, occ_kind, GeoOf<CK>::FTY);
    k_prolong_postsmooth<CK, VT, VTc, DOT, FINE><<<P.grid, P.block, sizeof(PostRing<CK>), s>>>(
        P.g, gc, sm, (const VT*)e, (const VTc*)ec, (const VT*)r, (VT*)out, (const VT*)accum, w, sc, partials,
        P.nblocks, n_active);
}

// r2 = r - A e on a coarse fused level, with the smoother's operator (the
// records' betas and diagonal): the right-hand side of a W-cycle level's
// second visit.
template <int CK, class VT>
__global__ void __launch_bounds__(TILE_THREADS) k_level_residual(Grid3 g, const void* __restrict__ sm_v,
                                                                 const VT* __restrict__ r, const VT* __restrict__ e,
                                                                 VT* __restrict__ r2, const Scalars* sc) {
    if (sc->converged) return;
    using CT = typename CoefStore<CK>::T;
    const CT* sm = reinterpret_cast<const CT*>(sm_v);
    const int x = blockIdx.x * TX + threadIdx.x, y = blockIdx.y * TY + threadIdx.y;
    if (x >= g.nx || y >= g.ny) return;
    const int z0 = blockIdx.z * g.zper, z1 = min(g.nz, z0 + g.zper);
    const long long sy = g.nx, sz = (long long)g.nx * g.ny;
    const int xm = wrap_or_neg(x - 1, g.nx, g.periodic & 1), xp = wrap_or_neg(x + 1, g.nx, g.periodic & 1);
    const int ym = wrap_or_neg(y - 1, g.ny, g.periodic & 2), yp = wrap_or_neg(y + 1, g.ny, g.periodic & 2);
    const int hx = split_x(x, g.nx), hxp = xp >= 0 ? split_x(xp, g.nx) : 0;
    for (int z = z0; z < z1; z++) {
        const long long i = x + sy * y + sz * z, is = i + (hx - x);
        const int zm = wrap_or_neg(z - 1, g.nz, g.periodic & 4), zp = wrap_or_neg(z + 1, g.nz, g.periodic & 4);
        const float4 own = unpack<CK>(sm[is]);
        const float bxh = xp >= 0 ? unpack<CK>(sm[is + (hxp - hx)]).x : 0.f;
        const float byh = yp >= 0 ? unpack<CK>(sm[is + (yp - y) * sy]).y : 0.f;
        const float bzh = zp >= 0 ? unpack<CK>(sm[is + (zp - z) * sz]).z : 0.f;
        float nsum = 0.f;
        nsum = fmaf(own.x, xm >= 0 ? to_f(e[i + (xm - x)]) : 0.f, nsum);
        nsum = fmaf(bxh, xp >= 0 ? to_f(e[i + (xp - x)]) : 0.f, nsum);
        nsum = fmaf(own.y, ym >= 0 ? to_f(e[i + (ym - y) * sy]) : 0.f, nsum);
        nsum = fmaf(byh, yp >= 0 ? to_f(e[i + (yp - y) * sy]) : 0.f, nsum);
        nsum = fmaf(own.z, zm >= 0 ? to_f(e[i + (zm - z) * sz]) : 0.f, nsum);
        nsum = fmaf(bzh, zp >= 0 ? to_f(e[i + (zp - z) * sz]) : 0.f, nsum);
        r2[i] = from_f<VT>(to_f(r[i]) - (own.w * to_f(e[i]) - nsum));
    }
}

// The coarse-grid correction of level l >= 1 for its right-hand side lv[l].r:
// fused passes on fused levels (two visits on W-cycle levels, the second on
// the residual of the first), the per-level / bottom kernels below.  Returns
// the buffer that holds the correction.
template <int CK, class VT>
static const void* fused_solve_level(const MGPlan& P, int l, double* partials, long long n_active, cudaStream_t s) {
    if (l >= P.fused_levels) {
        mg_vcycle_from(P, l, s);
        return P.lv[l].e;
    }
    const MGLevel &L = P.lv[l], &C = P.lv[l + 1];
    auto visit = [&](const void* rhs, void* out, const void* accum) {
        pre_impl<CK, VT, VT, false, false>(L.L.g, C.L.g, L.sm, rhs, nullptr, nullptr, L.e, C.r, P.sc, partials,
                                           O_PRE_COARSE, s);
        const void* ec = fused_solve_level<CK, VT>(P, l + 1, partials, n_active, s);
        post_impl<CK, VT, VT, false, false>(L.L.g, C.L.g, L.sm, L.e, ec, rhs, out, accum, P.prolong, P.sc, partials,
                                            n_active, O_POST_COARSE, s);
    };
    visit(L.r, L.eo, nullptr);
    if (P.w_from > 0 && l >= P.w_from && l <= P.w_to) {
        k_level_residual<CK, VT><<<L.L.grid, L.L.block, 0, s>>>(L.L.g, L.sm, (const VT*)L.r, (const VT*)L.eo,
                                                               (VT*)L.r2, P.sc);
        visit(L.r2, L.eo2, L.eo);
        return L.eo2;
    }
    return L.eo;
}

template <int CK, class VT>
static void vcycle_fused_impl(const MGPlan& P, const float* r_in, const float* q, float* r_out, bool update,
                              double* partials, long long n_active, cudaStream_t s) {
    if (update)
        pre_impl<CK, float, VT, true, true>(P.lv[0].L.g, P.lv[1].L.g, P.lv[0].sm, r_in, q, r_out, P.e0, P.lv[1].r,
                                            P.sc, partials, CK == 0 ? O_PRE_F32_UPD : O_PRE_LO_UPD, s);
    else
        pre_impl<CK, float, VT, false, true>(P.lv[0].L.g, P.lv[1].L.g, P.lv[0].sm, r_in, nullptr, nullptr, P.e0,
                                             P.lv[1].r, P.sc, partials, CK == 0 ? O_PRE_F32 : O_PRE_LO, s);
    const void* ec1 = fused_solve_level<CK, VT>(P, 1, partials, n_active, s);
    post_impl<CK, float, VT, true, true>(P.lv[0].L.g, P.lv[1].L.g, P.lv[0].sm, P.e0, ec1, update ? r_out : r_in,
                                         P.lv[0].e, nullptr, P.prolong, P.sc, partials, n_active,
                                         CK == 0 ? O_POST_F32 : O_POST_LO, s);
}

void mg_vcycle_fused(const MGPlan& P, const float* r_in, const float* q, float* r_out, bool update, double* partials,
                     long long n_active, cudaStream_t s) {
    if (P.precision == 1) vcycle_fused_impl<1, __half>(P, r_in, q, r_out, update, partials, n_active, s);
    else if (P.precision == 2) vcycle_fused_impl<2, __nv_bfloat16>(P, r_in, q, r_out, update, partials, n_active, s);
    else vcycle_fused_impl<0, float>(P, r_in, q, r_out, update, partials, n_active, s);
}

template <int CK>
static void records_impl(const MGPlan& P, cudaStream_t s) {
    for (int l = 0; l < P.fused_levels; l++) {
        const MGLevel& L = P.lv[l];
        const void* coef = CK == 0 ? (const void*)L.coef32 : L.coef_lo;
        k_smoother_records<CK><<<L.L.grid, L.L.block, 0, s>>>(L.L.g, coef, L.sm);
    }
}
void mg_smoother_records(const MGPlan& P, cudaStream_t s) {
    if (P.precision == 1) records_impl<1>(P, s);
    else if (P.precision == 2) records_impl<2>(P, s);
    else records_impl<0>(P, s);
}

// The coarse-grid correction of one V-cycle (level 1 and below), for
// measurement.
void mg_fused_coarse(const MGPlan& P, double* partials, long long n_active, cudaStream_t s) {
    if (P.fused_levels < 1 || P.nlevels < 2) return;
    if (P.precision == 1) (void)fused_solve_level<1, __half>(P, 1, partials, n_active, s);
    else if (P.precision == 2) (void)fused_solve_level<2, __nv_bfloat16>(P, 1, partials, n_active, s);
    else (void)fused_solve_level<0, float>(P, 1, partials, n_active, s);
}

// Single passes, for measurement.
void mg_fused_pre(const MGPlan& P, const float* r_in, const float* q, float* r_out, double* partials,
                  cudaStream_t s) {
    const Grid3 &g = P.lv[0].L.g, &gc = P.lv[1].L.g;
    const void* sm = P.lv[0].sm;
    if (P.precision == 1)
        pre_impl<1, float, __half, true, true>(g, gc, sm, r_in, q, r_out, P.e0, P.lv[1].r, P.sc, partials, O_PRE_LO_UPD, s);
    else if (P.precision == 2)
        pre_impl<2, float, __nv_bfloat16, true, true>(g, gc, sm, r_in, q, r_out, P.e0, P.lv[1].r, P.sc, partials,
                                                      O_PRE_LO_UPD, s);
    else
        pre_impl<0, float, float, true, true>(g, gc, sm, r_in, q, r_out, P.e0, P.lv[1].r, P.sc, partials, O_PRE_F32_UPD,
                                              s);
}
void mg_fused_post(const MGPlan& P, const float* r, double* partials, long long n_active, cudaStream_t s) {
    const Grid3 &g = P.lv[0].L.g, &gc = P.lv[1].L.g;
    const void* sm = P.lv[0].sm;
    const void* ec1 = (1 < P.fused_levels) ? P.lv[1].eo : P.lv[1].e;
    if (P.precision == 1)
        post_impl<1, float, __half, true, true>(g, gc, sm, P.e0, ec1, r, P.lv[0].e, nullptr, P.prolong, P.sc, partials,
                                                n_active, O_POST_LO, s);
    else if (P.precision == 2)
        post_impl<2, float, __nv_bfloat16, true, true>(g, gc, sm, P.e0, ec1, r, P.lv[0].e, nullptr, P.prolong, P.sc,
                                                       partials, n_active, O_POST_LO, s);
    else
        post_impl<0, float, float, true, true>(g, gc, sm, P.e0, ec1, r, P.lv[0].e, nullptr, P.prolong, P.sc, partials,
                                               n_active, O_POST_F32, s);
}

template <int CK, class VT, class VTc, bool UPDATE, bool FINE>
static cudaError_t prep_pre(int kind) {
    const void* fn = (const void*)k_presmooth_restrict<CK, VT, VTc, UPDATE, FINE>;
    const size_t bytes = sizeof(PreRing<CK>);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess && kind >= 0) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&f_occ[kind], fn, GeoOf<CK>::FT, bytes);
    return e;
}
template <int CK, class VT, class VTc, bool DOT, bool FINE>
static cudaError_t prep_post(int kind) {
    const void* fn = (const void*)k_prolong_postsmooth<CK, VT, VTc, DOT, FINE>;
    const size_t bytes = sizeof(PostRing<CK>);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess && kind >= 0) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&f_occ[kind], fn, GeoOf<CK>::FT, bytes);
    return e;
}

cudaError_t fused_prepare_attributes() {
    cudaError_t e = cudaSuccess;
    int dev = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&f_sms, cudaDevAttrMultiProcessorCount, dev);
#define PREP(x) \
    if (e == cudaSuccess) e = (x)
    PREP((prep_pre<0, float, float, false, true>(O_PRE_F32)));
    PREP((prep_pre<0, float, float, true, true>(O_PRE_F32_UPD)));
    PREP((prep_pre<1, float, __half, false, true>(O_PRE_LO)));
    PREP((prep_pre<1, float, __half, true, true>(O_PRE_LO_UPD)));
    PREP((prep_pre<2, float, __nv_bfloat16, false, true>(-1)));
    PREP((prep_pre<2, float, __nv_bfloat16, true, true>(-1)));
    PREP((prep_pre<0, float, float, false, false>(-1)));
    PREP((prep_pre<1, __half, __half, false, false>(O_PRE_COARSE)));
    PREP((prep_pre<2, __nv_bfloat16, __nv_bfloat16, false, false>(-1)));
    PREP((prep_post<0, float, float, true, true>(O_POST_F32)));
    PREP((prep_post<1, float, __half, true, true>(O_POST_LO)));
    PREP((prep_post<2, float, __nv_bfloat16, true, true>(-1)));
    PREP((prep_post<0, float, float, false, false>(-1)));
    PREP((prep_post<1, __half, __half, false, false>(O_POST_COARSE)));
    PREP((prep_post<2, __nv_bfloat16, __nv_bfloat16, false, false>(-1)));
#undef PREP
    if (e == cudaSuccess) e = tma_prepare_attributes();
    return e;
}

}  // namespace mhdproj
