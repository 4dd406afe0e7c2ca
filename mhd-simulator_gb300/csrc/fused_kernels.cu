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
// Both march a 64 x 8 (x, y) tile along z.  The stages of one pass run as a
// pipeline over planes: the pre-smoothing pass forms the residual and the red
// values of plane z, the black values of plane z-1 and the restricted
// residual of plane z-2 in the same step, so every input plane is read from
// HBM once.  A stage needs its neighbours' results, so each stage runs on a
// region one cell wider than the next: the red values cover the tile with a
// 2-cell halo, the black values a 1-cell halo, the residual the tile itself.
// Halo cells are recomputed by both neighbouring tiles from the same inputs
// in the same order, so the values agree bit for bit.  The smoother records
// are staged in shared memory with zero-filling 16-byte cp.async one plane
// ahead of the red stage (a staged row spans x0-4 .. x0+67, so every copy is
// a 16-byte-aligned group of records); the vector inputs of the red stage go
// to registers one plane ahead.  Three barriers per plane.
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
#include "staged.cuh"

namespace mhdproj {

namespace {
using namespace staged;

constexpr int PX = 2 * TX;       // 64 cells per tile row
constexpr int FTY = 8;           // tile rows (one thread row per tile row)
constexpr int FT = TX * FTY;     // 256 threads per block
constexpr int XO = 4;            // staged rows start at x0 - XO
constexpr int RW = PX + 2 * XO;  // 72 staged columns: x0-4 .. x0+67
constexpr int HW = RW / 2;       // 36 columns per half row (even x, then odd x)
constexpr int RH = FTY + 4;      // vector rows:  y0-2 .. y0+FTY+1
constexpr int CH = FTY + 5;      // record rows:  y0-2 .. y0+FTY+2
constexpr int RP = (PX + 4) / 2; // 34 pairs of the 2-halo region (x0-2 .. x0+65)
constexpr int NRED = RH * RP;    // 408 red-stage pair tasks
constexpr int NBLK = (FTY + 2) * RP;  // 340 black-stage pair tasks (rows y0-1 .. y0+FTY)
static_assert(NRED <= 2 * FT && NBLK <= 2 * FT, "two tasks per thread");

template <class VT> __device__ __forceinline__ float2 ld2(const VT* p);
template <> __device__ __forceinline__ float2 ld2<float>(const float* p) { return *reinterpret_cast<const float2*>(p); }
template <> __device__ __forceinline__ float2 ld2<__half>(const __half* p) {
    return __half22float2(*reinterpret_cast<const __half2*>(p));
}
template <> __device__ __forceinline__ float2 ld2<__nv_bfloat16>(const __nv_bfloat16* p) {
    return __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(p));
}
template <class VT> __device__ __forceinline__ void st2(VT* p, float2 v);
template <> __device__ __forceinline__ void st2<float>(float* p, float2 v) { *reinterpret_cast<float2*>(p) = v; }
template <> __device__ __forceinline__ void st2<__half>(__half* p, float2 v) {
    *reinterpret_cast<__half2*>(p) = __floats2half2_rn(v.x, v.y);
}
template <> __device__ __forceinline__ void st2<__nv_bfloat16>(__nv_bfloat16* p, float2 v) {
    *reinterpret_cast<__nv_bfloat162*>(p) = __floats2bfloat162_rn(v.x, v.y);
}
// Pairs of consecutive cells as loaded from a vector field, kept in the load
// type until the stage that uses them (a conversion right after the load
// would wait for the load).
template <class VT> struct Raw2 { using T = float2; };
template <> struct Raw2<__half> { using T = __half2; };
template <> struct Raw2<__nv_bfloat16> { using T = __nv_bfloat162; };
__device__ __forceinline__ void zero2(float2& v) { v = make_float2(0.f, 0.f); }
__device__ __forceinline__ void zero2(__half2& v) { v = __float2half2_rn(0.f); }
__device__ __forceinline__ void zero2(__nv_bfloat162& v) { v = __float2bfloat162_rn(0.f); }
template <class VT>
__device__ __forceinline__ typename Raw2<VT>::T ldg_pair(const VT* p, bool ok) {
    using R = typename Raw2<VT>::T;
    R v;
    if (ok) v = __ldg(reinterpret_cast<const R*>(p));
    else zero2(v);
    return v;
}
__device__ __forceinline__ float2 cvt2(const float2& v) { return v; }
__device__ __forceinline__ float2 cvt2(const __half2& v) { return __half22float2(v); }
__device__ __forceinline__ float2 cvt2(const __nv_bfloat162& v) { return __bfloat1622float2(v); }
template <class VT>
__device__ __forceinline__ VT ldg_one(const VT* p, bool ok) {
    return ok ? __ldg(p) : from_f<VT>(0.f);
}

// A thread's share of one plane's record copies, resolved once per block:
// two (8-byte records) or four (16-byte records) 16-byte copies of the
// record rows (13 rows x 2 half rows x 36 records).  A copy of two 8-byte
// records covers cells x and x+2 of a four-cell group, so both exist or
// neither does (nx is a multiple of 4).
template <int CK>
struct RecordFetch {
    using CT = typename CoefStore<CK>::T;
    static constexpr int RPC = (CK == 0) ? 1 : 2;  // records per 16-byte copy
    static constexpr int NCT = (CK == 0) ? 4 : 2;
    static constexpr int PER = HW / RPC;           // copies per half row
    static constexpr int NCTOT = CH * 2 * PER;
    static_assert(NCTOT <= NCT * FT, "record copies per thread");
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

// Shared-memory planes are [rows][2][HW]: each staged row holds its even-x
// cells, then its odd-x cells, so the cells of one colour in a row are
// contiguous.  A cell in half h at offset o has its x-1 neighbour at
// xminus(o, h) and its x+1 neighbour one further.
__device__ __forceinline__ int xminus(int o, int h) { return h ? o - HW : o + HW - 1; }

// The smoother records in HBM use the same split along whole grid rows: row
// (y, z) holds its nx/2 even-x records, then its nx/2 odd-x records, so a
// staged half row is one contiguous run.  Position of column x in its row:
__device__ __forceinline__ int split_x(int x, int nx) { return (x & 1) * (nx >> 1) + (x >> 1); }

// sum of beta * e over the six neighbours added to acc, in the per-cell
// kernels' order; *d = the cell's diagonal.  Offset o (half h) into the
// split planes; c/cn: record planes z, z+1; e/em/ep: correction planes z,
// z-1, z+1.
template <int CK, class CT>
__device__ __forceinline__ float gs_sum(const CT* c, const CT* cn, const float* e, const float* em, const float* ep,
                                        int o, int h, float acc, float* d) {
    const int xm = xminus(o, h);
    const float4 own = unpack<CK>(c[o]);
    const float bxh = unpack<CK>(c[xm + 1]).x;
    const float byh = unpack<CK>(c[o + RW]).y;
    const float bzh = unpack<CK>(cn[o]).z;
    acc = fmaf(own.x, e[xm], acc);
    acc = fmaf(bxh, e[xm + 1], acc);
    acc = fmaf(own.y, e[o - RW], acc);
    acc = fmaf(byh, e[o + RW], acc);
    acc = fmaf(own.z, em[o], acc);
    acc = fmaf(bzh, ep[o], acc);
    *d = own.w;
    return acc;
}

// A thread's pair tasks of the red / prolongation (2-halo) and black
// (1-halo) stages, resolved once per block: split-plane offsets of the pair's
// even cell (the odd cell is HW further), the colour parity of its row, the pair's in-plane offset in the grid
// (wrapped on periodic axes) and whether it exists, and for tasks on the tile
// the unwrapped in-plane offset (-1 otherwise).  Black tasks at the region's
// x edges update only the member inside the 1-halo.
struct PairTasks {
    int roff[2], rpar[2], rown[2], goff[2];
    bool gok[2];
    int boff[2], bpar[2], bedge[2];
    __device__ __forceinline__ PairTasks(const Grid3& g, int x0, int y0, int t) {
        const bool px = g.periodic & 1, py = g.periodic & 2;
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int k = t + u * FT;
            roff[u] = -1;
            rpar[u] = 0;
            rown[u] = -1;
            goff[u] = 0;
            gok[u] = false;
            if (k < NRED) {
                const int row = k / RP, pc = k - row * RP;
                roff[u] = row * RW + 1 + pc;
                rpar[u] = (y0 - 2 + row) & 1;
                const int gx = x0 - 2 + 2 * pc, gy = y0 - 2 + row;
                if (row >= 2 && row < FTY + 2 && pc >= 1 && pc <= TX && gx < g.nx && gy < g.ny) rown[u] = gx + g.nx * gy;
                bool okx, oky;
                const int sx = axis_src(gx, g.nx, px, &okx);
                const int sy = axis_src(gy, g.ny, py, &oky);
                gok[u] = okx && oky;
                goff[u] = gok[u] ? sx + g.nx * sy : 0;
            }
            boff[u] = -1;
            bpar[u] = 0;
            bedge[u] = 0;
            if (k < NBLK) {
                const int rr = k / RP, pc = k - rr * RP, row = rr + 1;
                boff[u] = row * RW + 1 + pc;
                bpar[u] = (1 + y0 - 2 + row) & 1;
                bedge[u] = pc == 0 ? 1 : (pc == RP - 1 ? 2 : 0);
            }
        }
    }
    // red member (0 or 1) of red task u at plane z
    __device__ __forceinline__ int red(int u, int z) const { return (rpar[u] + z) & 1; }
    // black member (0 or 1) of black task u at plane z, or -1 when it lies
    // outside the 1-halo
    __device__ __forceinline__ int black(int u, int z) const {
        const int m = (bpar[u] + z) & 1;
        if ((bedge[u] == 1 && m == 0) || (bedge[u] == 2 && m == 1)) return -1;
        return m;
    }
};

// Plane rings in shared memory.  A step handles planes zA (red /
// prolongation stage), zA-1 (black stage) and zA-2 (tile stage) and stages
// the records of plane zA+1 for the next step; rings of 4 planes, so the z
// loop is unrolled four times and every slot is a compile-time offset.  The
// vector inputs go straight to registers, one plane ahead.  In the correction
// ring the black cells of the newest plane hold their right-hand side sigma r
// until the black stage replaces it by their value.
template <int CK>
struct PreRing {
    using CT = typename CoefStore<CK>::T;
    CT c[4][CH][RW];                 // records, planes zA-2 .. zA+1
    float er[4][RH][RW];             // correction, planes zA-3 .. zA
    float ypart[FTY][TX];
};
template <int CK>
struct PostRing {
    using CT = typename CoefStore<CK>::T;
    CT c[4][CH][RW];                 // records, planes zA-2 .. zA+1
    float ep[4][RH][RW];             // prolonged / smoothed correction, planes zA-3 .. zA
};
template <int N>
using Phase = std::integral_constant<int, N>;
template <int CK>
constexpr int fused_min_blocks() { return CK == 0 ? 3 : 4; }
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
__global__ void __launch_bounds__(FT, fused_min_blocks<CK>())
    k_presmooth_restrict(Grid3 g, Grid3 gc, const void* __restrict__ sm_v, const VT* __restrict__ rin,
                         const float* __restrict__ q, float* __restrict__ r_out, VT* __restrict__ e,
                         VTc* __restrict__ rc, Scalars* sc, double* partials, int nblocks) {
    if (sc->converged) return;
    using CT = typename CoefStore<CK>::T;
    using R2 = typename Raw2<VT>::T;
    const CT* sm = reinterpret_cast<const CT*>(sm_v);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto& S = *reinterpret_cast<PreRing<CK>*>(smem_raw);
    __shared__ double sh[FT / 32];
    const float sigma = FINE ? sc->sigma : 1.0f;
    const float alpha = UPDATE ? sc->alpha_f : 0.0f;
    const int x0 = blockIdx.x * PX, y0 = blockIdx.y * FTY;
    const int tx = threadIdx.x, ty = threadIdx.y, t = tx + TX * ty;
    const int z0 = blockIdx.z * g.zper, z1 = min(g.nz, z0 + g.zper);
    const RecordFetch<CK> F(g, x0, y0, t);
    const PairTasks T(g, x0, y0, t);
    const long long sxy = (long long)g.nx * g.ny;
    // ||r||^2 only steers the stop test and sigma: a per-thread FP32 sum,
    // FP64 across threads and blocks
    float rr_thread = 0.f;
    float part = 0.f;
    int rc_z = -1;  // coarse plane whose restriction awaits the row pair sum
    const int ox = x0 + 2 * tx, oy = y0 + ty;  // the thread's own pair
    const bool own_inside = ox < g.nx && oy < g.ny;
    const int oo = (ty + 2) * RW + XO / 2 + tx;  // split offset of its even cell
    const long long og = ox + (long long)g.nx * oy;
    R2 rv[2], rvn[2];
    float2 qv[2], qvn[2];
    // records of plane zz to ring slot c4 (cp.async), the red tasks' residual
    // (and q) of plane zz to registers
    auto fetch = [&](int zz, int c4, R2* rd, float2* qd) {
        bool okz;
        const long long pl = F.plane(zz, &okz);
        F.recs(&S.c[c4][0][0], sm, pl, okz);
        cp_commit();
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const bool ok = T.gok[u] && okz;
            rd[u] = ldg_pair<VT>(rin + pl + T.goff[u], ok);
            if (UPDATE) qd[u] = ok ? __ldg(reinterpret_cast<const float2*>(q + pl + T.goff[u])) : make_float2(0.f, 0.f);
        }
    };
    auto flush_rc = [&]() {
        if (rc_z >= 0 && own_inside && !(ty & 1)) {
            const float tot = S.ypart[ty][tx] + S.ypart[ty + 1][tx];
            rc[(ox >> 1) + (long long)gc.nx * ((oy >> 1) + (long long)gc.ny * rc_z)] = from_f<VTc>(0.25f * tot);
        }
        rc_z = -1;
    };
    auto step = [&](auto ph, int zA) {
        constexpr int P = decltype(ph)::value;
        cp_wait<0>();
        __syncthreads();
        fetch(zA + 1, (P + 1) & 3, rvn, UPDATE ? qvn : nullptr);
        flush_rc();
        // ---- red stage: plane zA over the 2-halo region
        {
            const CT* C = &S.c[P][0][0];
            float* ER = &S.er[P][0][0];
            const bool zin = zA >= z0 && zA < z1;
            float* rplane = UPDATE ? r_out + sxy * zA : nullptr;
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const int o = T.roff[u];
                if (o < 0) break;
                float2 rn = cvt2(rv[u]);
                if (UPDATE) rn = make_float2(fmaf(-alpha, qv[u].x, rn.x), fmaf(-alpha, qv[u].y, rn.y));
                const int m = T.red(u, zA);
                const float d = unpack<CK>(C[o + m * HW]).w;
                const float ev = d > 0.f ? __fdividef(sigma * (m ? rn.y : rn.x), d) : 0.f;
                ER[o] = m ? sigma * rn.x : ev;
                ER[o + HW] = m ? ev : sigma * rn.y;
                if (UPDATE && zin && T.rown[u] >= 0) {
                    *reinterpret_cast<float2*>(rplane + T.rown[u]) = rn;
                    rr_thread = fmaf(rn.x, rn.x, fmaf(rn.y, rn.y, rr_thread));
                }
            }
        }
        __syncthreads();
        // ---- black stage: plane zA-1 over the 1-halo region, in place
        const int zB = zA - 1;
        if (zB >= z0 - 1) {
            const CT* C = &S.c[(P + 3) & 3][0][0];
            const CT* CN = &S.c[P][0][0];
            float* E = &S.er[(P + 3) & 3][0][0];
            const float* EM = &S.er[(P + 2) & 3][0][0];
            const float* EP = &S.er[P][0][0];
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const int h = T.black(u, zB);
                if (h < 0) continue;
                const int o = T.boff[u] + h * HW;
                float d;
                const float s = gs_sum<CK>(C, CN, E, EM, EP, o, h, E[o], &d);
                E[o] = d > 0.f ? __fdividef(s, d) : 0.f;
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
            const int m = (y0 + ty + zC) & 1;  // red member of the own pair
            float d;
            part += gs_sum<CK>(C, CN, E, EM, EP, oo + m * HW, m, 0.f, &d);
            if (own_inside) st2<VT>(e + (og + sxy * zC), make_float2(E[oo], E[oo + HW]));
            if (((zC - z0) & 1) || zC + 1 == z1) {
                // the row pair sum is formed after the next barrier
                S.ypart[ty][tx] = part;
                rc_z = zC >> 1;
                part = 0.f;
            }
        }
#pragma unroll
        for (int u = 0; u < 2; u++) {
            rv[u] = rvn[u];
            if (UPDATE) qv[u] = qvn[u];
        }
    };
    const int zs = z0 - 2, zend = z1 + 1;  // red stage over zs .. zend
    fetch(zs, 0, rv, UPDATE ? qv : nullptr);
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
__global__ void __launch_bounds__(FT, fused_min_blocks<CK>())
    k_prolong_postsmooth(Grid3 g, Grid3 gc, const void* __restrict__ sm_v, const VT* __restrict__ e,
                         const VTc* __restrict__ ec, const VT* __restrict__ r, VT* __restrict__ out,
                         const VT* __restrict__ accum, float w, Scalars* sc, double* partials, int nblocks,
                         long long n_active) {
    if (sc->converged) return;
    using CT = typename CoefStore<CK>::T;
    using R2 = typename Raw2<VT>::T;
    const CT* sm = reinterpret_cast<const CT*>(sm_v);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto& S = *reinterpret_cast<PostRing<CK>*>(smem_raw);
    __shared__ double sh[FT / 32];
    const float sigma = FINE ? sc->sigma : 1.0f;
    const float is = FINE ? sc->inv_sigma : 1.0f;
    const int x0 = blockIdx.x * PX, y0 = blockIdx.y * FTY;
    const int tx = threadIdx.x, ty = threadIdx.y, t = tx + TX * ty;
    const int z0 = blockIdx.z * g.zper, z1 = min(g.nz, z0 + g.zper);
    const RecordFetch<CK> F(g, x0, y0, t);
    const PairTasks T(g, x0, y0, t);
    const long long sxy = (long long)g.nx * g.ny;
    // coarse parents of the red-stage pairs: in-plane offsets
    int pofs[2];
    {
        const bool px = g.periodic & 1, py = g.periodic & 2;
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int k = t + u * FT;
            pofs[u] = 0;
            if (k < NRED) {
                const int row = k / RP, pc = k - row * RP;
                bool okx, oky;
                const int sx = axis_src(x0 - 2 + 2 * pc, g.nx, px, &okx);
                const int sy = axis_src(y0 - 2 + row, g.ny, py, &oky);
                pofs[u] = (okx && oky) ? (sx >> 1) + gc.nx * (sy >> 1) : 0;
            }
        }
    }
    const long long csxy = (long long)gc.nx * gc.ny;
    Acc acc;
    const int ox = x0 + 2 * tx, oy = y0 + ty;
    const bool own_inside = ox < g.nx && oy < g.ny;
    const int oo = (ty + 2) * RW + XO / 2 + tx;
    const long long og = ox + (long long)g.nx * oy;
    // registers of plane zA (current) and zA+1 (next): the pre-smoothed
    // correction of the red-stage pairs, their black member's right-hand
    // side, the coarse parents, and the own pair's right-hand side of the
    // next tile plane
    R2 eov[2], eon[2];
    VT rbv[2], rbn[2];
    VTc pcv[2], pcn[2];
    R2 rov, ron;
    auto fetch = [&](int zz, int c4, R2* eo, VT* rb, VTc* pc, R2& ro) {
        bool okz;
        const int sz = axis_src(zz, g.nz, (g.periodic & 4) != 0, &okz);
        const long long pl = (long long)sz * sxy, cpl = (long long)(sz >> 1) * csxy;
        F.recs(&S.c[c4][0][0], sm, pl, okz);
        cp_commit();
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const bool ok = T.gok[u] && okz;
            eo[u] = ldg_pair<VT>(e + pl + T.goff[u], ok);
            rb[u] = ldg_one<VT>(r + pl + T.goff[u] + (1 - T.red(u, zz)), ok);
            pc[u] = ldg_one<VTc>(ec + cpl + pofs[u], ok);
        }
        const int zt = zz - 2;  // tile plane of the next step
        ro = ldg_pair<VT>(r + og + sxy * zt, own_inside && zt >= z0 && zt < z1);
    };
    auto step = [&](auto ph, int zA) {
        constexpr int P = decltype(ph)::value;
        cp_wait<0>();
        __syncthreads();
        fetch(zA + 1, (P + 1) & 3, eon, rbn, pcn, ron);
        // ---- prolongation: plane zA over the 2-halo region
        {
            float* EP = &S.ep[P][0][0];
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const int o = T.roff[u];
                if (o < 0) break;
                const float2 ev = cvt2(eov[u]);
                const float cv = to_f(pcv[u]);
                const float rb = sigma * to_f(rbv[u]);
                const bool m = T.red(u, zA);
                EP[o] = m ? rb : fmaf(w, cv, ev.x);
                EP[o + HW] = m ? fmaf(w, cv, ev.y) : rb;
            }
        }
        __syncthreads();
        // ---- black half-step: plane zA-1 over the 1-halo region, in place
        const int zB = zA - 1;
        if (zB >= z0 - 1) {
            const CT* C = &S.c[(P + 3) & 3][0][0];
            const CT* CN = &S.c[P][0][0];
            float* E = &S.ep[(P + 3) & 3][0][0];
            const float* EM = &S.ep[(P + 2) & 3][0][0];
            const float* EP = &S.ep[P][0][0];
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const int h = T.black(u, zB);
                if (h < 0) continue;
                const int o = T.boff[u] + h * HW;
                float d;
                const float s = gs_sum<CK>(C, CN, E, EM, EP, o, h, E[o], &d);
                E[o] = d > 0.f ? __fdividef(s, d) : 0.f;
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
            const int m = (y0 + ty + zC) & 1;  // the pair member of colour 0
            const float2 rv = cvt2(rov);
            float d;
            const float s = gs_sum<CK>(C, CN, E, EM, EP, oo + m * HW, m, sigma * (m ? rv.y : rv.x), &d);
            const float zr = d > 0.f ? __fdividef(s, d) : 0.f;
            const float zb = E[oo + (1 - m) * HW];
            float2 zv = m ? make_float2(zb, zr) : make_float2(zr, zb);
            if (own_inside) {
                if (accum) {  // out = accum + z (second W-cycle visit)
                    const float2 a = ld2<VT>(accum + og + sxy * zC);
                    zv = make_float2(a.x + zv.x, a.y + zv.y);
                }
                st2<VT>(out + og + sxy * zC, zv);
                if (DOT) {
                    acc.add_prod(rv.x, zv.x * is);
                    acc.add_prod(rv.y, zv.y * is);
                }
            }
        }
#pragma unroll
        for (int u = 0; u < 2; u++) {
            eov[u] = eon[u];
            rbv[u] = rbn[u];
            pcv[u] = pcn[u];
        }
        rov = ron;
    };
    const int zs = z0 - 2, zend = z1 + 1;
    fetch(zs, 0, eov, rbv, pcv, rov);
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
// run also computes two planes below and above it.
Launch fused_launch(const Grid3& g0, int occ_kind) {
    Launch P;
    P.g = g0;
    P.block = dim3(TX, FTY, 1);
    const int gx = (g0.nx + PX - 1) / PX, gy = (g0.ny + FTY - 1) / FTY, nz = g0.nz;
    const int tiles = gx * gy;
    const int cap = (f_sms > 0 ? f_sms : 152) * (f_occ[occ_kind] > 0 ? f_occ[occ_kind] : 1);
    int best_zper = nz + (nz & 1), best_zc = 1;
    double best = -1.0;
    for (int zc = 1; zc <= nz; zc++) {
        int zper = (nz + zc - 1) / zc;
        if (zper & 1) zper++;
        if (zper < 4 && zc > 1) break;
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
    const Launch P = fused_launch(g, occ_kind);
    k_presmooth_restrict<CK, VT, VTc, UPDATE, FINE><<<P.grid, P.block, sizeof(PreRing<CK>), s>>>(
        P.g, gc, sm, (const VT*)rin, q, r_out, (VT*)e, (VTc*)rc, sc, partials, P.nblocks);
}
template <int CK, class VT, class VTc, bool DOT, bool FINE>
static void post_impl(const Grid3& g, const Grid3& gc, const void* sm, const void* e, const void* ec, const void* r,
                      void* out, const void* accum, float w, Scalars* sc, double* partials, long long n_active,
                      int occ_kind, cudaStream_t s) {
    const Launch P = fused_launch(g, occ_kind);
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
    if (e == cudaSuccess && kind >= 0) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&f_occ[kind], fn, FT, bytes);
    return e;
}
template <int CK, class VT, class VTc, bool DOT, bool FINE>
static cudaError_t prep_post(int kind) {
    const void* fn = (const void*)k_prolong_postsmooth<CK, VT, VTc, DOT, FINE>;
    const size_t bytes = sizeof(PostRing<CK>);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess && kind >= 0) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&f_occ[kind], fn, FT, bytes);
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
    return e;
}

}  // namespace mhdproj
