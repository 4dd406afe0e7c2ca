// mg_kernels.cu -- the GB300 solver's multigrid preconditioner.
//
// Hierarchy: the reference's 2x2x2 aggregation (src/fluid/multigrid.rs:25-65:
// halve with ceiling until every extent is <= 4) with piecewise-constant
// prolongation P and the Galerkin coarse graph P^T A P (multigrid.wgsl:50-65:
// crossing edges summed, reactions summed, internal edges dropped).  Each
// level is stored scaled by a power of two so FP16 fields stay in range:
//   coarse coefficients   A_{l+1} = 1/4 P^T A_l P
//   restriction           r_{l+1} = 1/4 P^T (r_l - A_l e_l)
//   prolongation          e_l    += w P e_{l+1}          (w = 2 by default)
// which is a coarse correction of w P (P^T A P)^-1 P^T.  Smoothing is one
// red-black Gauss-Seidel sweep before (red, black) and after (black, red) the
// coarse correction, and the coarsest level (every extent <= 4, at most 64
// cells) is solved exactly with a dense inverse, so the V-cycle is a fixed
// symmetric operator.
// Level fields (coefficients and vectors of levels >= 1, the fine smoother's
// coefficients) are FP32, FP16 or BF16; arithmetic is FP32.
#include <algorithm>
#include <cstdlib>
#include <functional>

#include "kernels.h"
#include "staged.cuh"

namespace mhdproj {

#define TILE_BEGIN(G)                                      \
    const int x = blockIdx.x * TX + threadIdx.x;           \
    const int y = blockIdx.y * TY + threadIdx.y;           \
    const bool in_xy = x < (G).nx && y < (G).ny;           \
    const int z0 = blockIdx.z * (G).zper;                  \
    const int z1 = min((G).nz, z0 + (G).zper);             \
    for (int z = z0; z < z1; z++)

template <int CK> __device__ __forceinline__ float4 ldc(const void* p, int i);
template <> __device__ __forceinline__ float4 ldc<0>(const void* p, int i) {
    return load_coef(reinterpret_cast<const float4*>(p), i);
}
template <> __device__ __forceinline__ float4 ldc<1>(const void* p, int i) {
    return load_coef_h(reinterpret_cast<const uint2*>(p), i);
}
template <> __device__ __forceinline__ float4 ldc<2>(const void* p, int i) {
    return load_coef_b(reinterpret_cast<const uint2*>(p), i);
}

struct Stencil {
    int xm, xp, ym, yp, zm, zp;
    float bxl, byl, bzl, bxh, byh, bzh, react, diag;
};
template <int CK>
__device__ __forceinline__ Stencil stencil(const Grid3& g, const void* coef, int x, int y, int z) {
    Stencil s;
    const int sy = g.nx, sz = g.nx * g.ny;
    const int i = x + sy * y + sz * z;
    int c;
    c = wrap_or_neg(x - 1, g.nx, g.periodic & 1); s.xm = c < 0 ? -1 : i + (c - x);
    c = wrap_or_neg(x + 1, g.nx, g.periodic & 1); s.xp = c < 0 ? -1 : i + (c - x);
    c = wrap_or_neg(y - 1, g.ny, g.periodic & 2); s.ym = c < 0 ? -1 : i + (c - y) * sy;
    c = wrap_or_neg(y + 1, g.ny, g.periodic & 2); s.yp = c < 0 ? -1 : i + (c - y) * sy;
    c = wrap_or_neg(z - 1, g.nz, g.periodic & 4); s.zm = c < 0 ? -1 : i + (c - z) * sz;
    c = wrap_or_neg(z + 1, g.nz, g.periodic & 4); s.zp = c < 0 ? -1 : i + (c - z) * sz;
    const float4 own = ldc<CK>(coef, i);
    s.bxl = own.x;
    s.byl = own.y;
    s.bzl = own.z;
    s.react = own.w;
    s.bxh = s.xp >= 0 ? ldc<CK>(coef, s.xp).x : 0.0f;
    s.byh = s.yp >= 0 ? ldc<CK>(coef, s.yp).y : 0.0f;
    s.bzh = s.zp >= 0 ? ldc<CK>(coef, s.zp).z : 0.0f;
    s.diag = ((s.bxl + s.bxh) + (s.byl + s.byh)) + ((s.bzl + s.bzh) + s.react);
    return s;
}
// sum of beta * e over the six neighbours
template <class VT>
__device__ __forceinline__ float neighbour_sum(const Stencil& s, const VT* e) {
    float acc = 0.0f;
    if (s.bxl != 0.0f) acc = fmaf(s.bxl, to_f(e[s.xm]), acc);
    if (s.bxh != 0.0f) acc = fmaf(s.bxh, to_f(e[s.xp]), acc);
    if (s.byl != 0.0f) acc = fmaf(s.byl, to_f(e[s.ym]), acc);
    if (s.byh != 0.0f) acc = fmaf(s.byh, to_f(e[s.yp]), acc);
    if (s.bzl != 0.0f) acc = fmaf(s.bzl, to_f(e[s.zm]), acc);
    if (s.bzh != 0.0f) acc = fmaf(s.bzh, to_f(e[s.zp]), acc);
    return acc;
}

template <int CK> __device__ __forceinline__ float ldc_x(const void* p, int i);
template <> __device__ __forceinline__ float ldc_x<0>(const void* p, int i) {
    return __ldg(reinterpret_cast<const float*>(p) + 4 * i);
}
template <> __device__ __forceinline__ float ldc_x<1>(const void* p, int i) {
    return __half2float(__ldg(reinterpret_cast<const __half*>(p) + 4 * i));
}
template <> __device__ __forceinline__ float ldc_x<2>(const void* p, int i) {
    return __bfloat162float(__ldg(reinterpret_cast<const __nv_bfloat16*>(p) + 4 * i));
}
template <int CK> __device__ __forceinline__ float ldc_y(const void* p, int i);
template <> __device__ __forceinline__ float ldc_y<0>(const void* p, int i) {
    return __ldg(reinterpret_cast<const float*>(p) + 4 * i + 1);
}
template <> __device__ __forceinline__ float ldc_y<1>(const void* p, int i) {
    return __half2float(__ldg(reinterpret_cast<const __half*>(p) + 4 * i + 1));
}
template <> __device__ __forceinline__ float ldc_y<2>(const void* p, int i) {
    return __bfloat162float(__ldg(reinterpret_cast<const __nv_bfloat16*>(p) + 4 * i + 1));
}

// One red-black Gauss-Seidel half-step on `color` cells.  ZERO: the first
// half-step from a zero correction (e = rhs/diag on color cells, 0 elsewhere).
// OUT: write color cells to `out` instead of in place (levels whose periodic
// extents are odd have same-colour neighbours across the wrap).  Each thread
// marches its column along z with the coefficient records at z, z+1 and the
// corrections at z-1, z+1 in registers, loading plane z+2 one step ahead.
template <int CK, class VT, bool FINE, bool ZERO, bool OUT>
__global__ void __launch_bounds__(TILE_THREADS) k_smooth(Grid3 g, const void* __restrict__ coef,
                                                         const VT* __restrict__ r, VT* e, VT* out, int color,
                                                         const Scalars* sc) {
    if (sc->converged) return;
    const float sigma = FINE ? sc->sigma : 1.0f;
    const int x = blockIdx.x * TX + threadIdx.x, y = blockIdx.y * TY + threadIdx.y;
    const int z0 = blockIdx.z * g.zper, z1 = min(g.nz, z0 + g.zper);
    if (x >= g.nx || y >= g.ny) return;
    const Column C(g, x, y);
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 cc = ldc<CK>(coef, C.at(z0));
    float4 cn = C.zexists(z0 + 1) ? ldc<CK>(coef, C.zat(z0 + 1)) : zero4;
    float em = 0.f, ec = 0.f, en = 0.f;
    if (!ZERO) {
        em = to_f(e[C.zat(z0 - 1)]);
        ec = to_f(e[C.at(z0)]);
        en = to_f(e[C.zat(z0 + 1)]);
    }
    for (int z = z0; z < z1; z++) {
        const int i = C.at(z);
        float4 cnn = zero4;
        float enn = 0.f;
        if (z + 1 < z1) {
            if (C.zexists(z + 2)) cnn = ldc<CK>(coef, C.zat(z + 2));
            if (!ZERO) enn = to_f(e[C.zat(z + 2)]);
        }
        if (((x + y + z) & 1) == color) {
            const float bxh = C.hxp ? ldc_x<CK>(coef, i + C.dxp) : 0.f;
            const float byh = C.hyp ? ldc_y<CK>(coef, i + C.dyp) : 0.f;
            const float d = ((cc.x + bxh) + (cc.y + byh)) + ((cc.z + cn.z) + cc.w);
            float val = 0.f;
            if (d > 0.f) {
                const float rhs = sigma * to_f(r[i]);
                if (ZERO) {
                    val = rhs / d;
                } else {
                    float acc = rhs;
                    acc = fmaf(cc.x, to_f(e[i + C.dxm]), acc);
                    acc = fmaf(bxh, to_f(e[i + C.dxp]), acc);
                    acc = fmaf(cc.y, to_f(e[i + C.dym]), acc);
                    acc = fmaf(byh, to_f(e[i + C.dyp]), acc);
                    acc = fmaf(cc.z, em, acc);
                    acc = fmaf(cn.z, en, acc);
                    val = acc / d;
                }
            }
            if (OUT) out[i] = from_f<VT>(val);
            else e[i] = from_f<VT>(val);
        } else if (ZERO) {
            e[i] = from_f<VT>(0.0f);
        }
        cc = cn;
        cn = cnn;
        if (!ZERO) {
            // Carry the values read before this half-step: a cell of this
            // colour is never the z-neighbour of another cell of this colour,
            // so its old value is only used when it is not updated.
            em = ec;
            ec = en;
            en = enn;
        }
    }
}
template <class VT>
__global__ void __launch_bounds__(TILE_THREADS) k_copy_color(Grid3 g, const VT* __restrict__ in, VT* __restrict__ e,
                                                             int color, const Scalars* sc) {
    if (sc->converged) return;
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        if (((x + y + z) & 1) != color) continue;
        const int i = x + g.nx * (y + g.ny * z);
        e[i] = in[i];
    }
}

// Residual of the children and restriction: rc[Q] = 1/4 sum (rhs - A e),
// launched over the fine grid with an even z run per block.  A thread forms
// the residual of its cell for two planes (the z pair), adds its x partner by
// a warp shuffle and its y partner through shared memory; the thread at the
// even (x, y) corner writes the coarse value.
template <int CK, class VTf, bool FINE, class VTc>
__global__ void __launch_bounds__(TILE_THREADS) k_restrict(Grid3 gf, Grid3 gc, const void* __restrict__ coef,
                                                           const VTf* __restrict__ r, const VTf* __restrict__ e,
                                                           VTc* __restrict__ rc, const Scalars* sc) {
    if (sc->converged) return;
    __shared__ float ypart[TY][TX];
    const float sigma = FINE ? sc->sigma : 1.0f;
    const int x = blockIdx.x * TX + threadIdx.x, y = blockIdx.y * TY + threadIdx.y;
    const int z0 = blockIdx.z * gf.zper, z1 = min(gf.nz, z0 + gf.zper);
    const bool inside = x < gf.nx && y < gf.ny;
    const Column C(gf, inside ? x : 0, inside ? y : 0);
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 cc = zero4, cn = zero4;
    float em = 0.f, ec = 0.f, en = 0.f;
    if (inside && z0 < z1) {
        cc = ldc<CK>(coef, C.at(z0));
        cn = C.zexists(z0 + 1) ? ldc<CK>(coef, C.zat(z0 + 1)) : zero4;
        em = to_f(e[C.zat(z0 - 1)]);
        ec = to_f(e[C.at(z0)]);
        en = to_f(e[C.zat(z0 + 1)]);
    }
    for (int z = z0; z < z1; z += 2) {
        float part = 0.f;
#pragma unroll
        for (int k = 0; k < 2; k++) {
            const int zz = z + k;
            if (inside && zz < z1) {
                const int i = C.at(zz);
                float4 cnn = zero4;
                float enn = 0.f;
                if (zz + 1 < z1) {
                    if (C.zexists(zz + 2)) cnn = ldc<CK>(coef, C.zat(zz + 2));
                    enn = to_f(e[C.zat(zz + 2)]);
                }
                const float bxh = C.hxp ? ldc_x<CK>(coef, i + C.dxp) : 0.f;
                const float byh = C.hyp ? ldc_y<CK>(coef, i + C.dyp) : 0.f;
                const float d = ((cc.x + bxh) + (cc.y + byh)) + ((cc.z + cn.z) + cc.w);
                float nsum = 0.f;
                nsum = fmaf(cc.x, to_f(e[i + C.dxm]), nsum);
                nsum = fmaf(bxh, to_f(e[i + C.dxp]), nsum);
                nsum = fmaf(cc.y, to_f(e[i + C.dym]), nsum);
                nsum = fmaf(byh, to_f(e[i + C.dyp]), nsum);
                nsum = fmaf(cc.z, em, nsum);
                nsum = fmaf(cn.z, en, nsum);
                part += sigma * to_f(r[i]) - (d * ec - nsum);
                cc = cn;
                cn = cnn;
                em = ec;
                ec = en;
                en = enn;
            }
        }
        part += __shfl_xor_sync(0xffffffffu, part, 1);
        ypart[threadIdx.y][threadIdx.x] = part;
        __syncthreads();
        if (inside && !(threadIdx.x & 1) && !(threadIdx.y & 1)) {
            const float tot = part + ypart[threadIdx.y + 1][threadIdx.x];
            rc[(x >> 1) + gc.nx * ((y >> 1) + gc.ny * (z >> 1))] = from_f<VTc>(0.25f * tot);
        }
        __syncthreads();
    }
}

template <class VTf, class VTc>
__global__ void __launch_bounds__(TILE_THREADS) k_prolong(Grid3 gf, Grid3 gc, VTf* __restrict__ e,
                                                          const VTc* __restrict__ ec, float w, const Scalars* sc) {
    if (sc->converged) return;
    const int x = blockIdx.x * TX + threadIdx.x, y = blockIdx.y * TY + threadIdx.y;
    const int z0 = blockIdx.z * gf.zper, z1 = min(gf.nz, z0 + gf.zper);
    if (x >= gf.nx || y >= gf.ny) return;
    const int sxy = gf.nx * gf.ny, base = x + gf.nx * y;
    const int cbase = (x >> 1) + gc.nx * (y >> 1), csxy = gc.nx * gc.ny;
    int z = z0;
    for (; z + 3 < z1; z += 4) {
        float ev[4], cv[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            ev[k] = to_f(e[base + (z + k) * sxy]);
            cv[k] = to_f(ec[cbase + ((z + k) >> 1) * csxy]);
        }
#pragma unroll
        for (int k = 0; k < 4; k++) e[base + (z + k) * sxy] = from_f<VTf>(fmaf(w, cv[k], ev[k]));
    }
    for (; z < z1; z++) {
        const int i = base + z * sxy;
        e[i] = from_f<VTf>(fmaf(w, to_f(ec[cbase + (z >> 1) * csxy]), to_f(e[i])));
    }
}

// Exact coarsest solve: e = Ainv * rhs (m <= 64).
template <class VT, bool FINE>
__global__ void k_coarse_solve(int m, const float* __restrict__ ainv, const VT* __restrict__ r, VT* __restrict__ e,
                               const Scalars* sc) {
    if (sc->converged) return;
    __shared__ float rhs[64];
    const float sigma = FINE ? sc->sigma : 1.0f;
    const int t = threadIdx.x;
    if (t < m) rhs[t] = sigma * to_f(r[t]);
    __syncthreads();
    if (t < m) {
        float s = 0.0f;
        for (int k = 0; k < m; k++) s = fmaf(ainv[t * m + k], rhs[k], s);
        e[t] = from_f<VT>(s);
    }
}

// Galerkin coarse graph of one level from the FP32 master of the finer one.
template <int CKLO>
__global__ void __launch_bounds__(TILE_THREADS) k_mg_build(Grid3 gf, Grid3 gc, const float4* __restrict__ cf,
                                                           float4* __restrict__ cc, void* __restrict__ lo) {
    TILE_BEGIN(gc) {
        if (!in_xy) continue;
        float c[4] = {0.f, 0.f, 0.f, 0.f};
        for (int dz = 0; dz < 2; dz++)
            for (int dy = 0; dy < 2; dy++)
                for (int dx = 0; dx < 2; dx++) {
                    const int cx = 2 * x + dx, cy = 2 * y + dy, cz = 2 * z + dz;
                    if (cx >= gf.nx || cy >= gf.ny || cz >= gf.nz) continue;
                    const int ci = cx + gf.nx * (cy + gf.ny * cz);
                    const float4 f = cf[ci];
                    c[3] += f.w;
                    const float fb[3] = {f.x, f.y, f.z};
                    const int cc3[3] = {cx, cy, cz}, n3[3] = {gf.nx, gf.ny, gf.nz}, q3[3] = {x, y, z};
#pragma unroll
                    for (int a = 0; a < 3; a++) {
                        const int l = wrap_or_neg(cc3[a] - 1, n3[a], gf.periodic & (1 << a));
                        if (l < 0) continue;
                        const float beta = fb[a];
                        if (beta == 0.0f) continue;
                        // The low neighbour differs from the child only along a.
                        if ((l >> 1) == q3[a]) continue;
                        c[a] += beta;
                    }
                }
        const float4 out = make_float4(c[0] * 0.25f, c[1] * 0.25f, c[2] * 0.25f, c[3] * 0.25f);
        const int Q = x + gc.nx * (y + gc.ny * z);
        cc[Q] = out;
        if (CKLO == 1) reinterpret_cast<uint2*>(lo)[Q] = pack_coef_h(out);
        if (CKLO == 2) reinterpret_cast<uint2*>(lo)[Q] = pack_coef_b(out);
    }
}

// Dense inverse of the coarsest operator (m <= 64 cells) in FP64, one column
// per block: every block assembles A, factors it A = L L^T (Cholesky; the
// operator is symmetric positive definite on the active cells) and solves
// L L^T x = e_b for its column b.  Rows of empty aggregates (diagonal 0) are
// identity rows during the factorisation and zero in the stored inverse.
// Spreading the columns over blocks spreads the FP64 work over SMs; each
// block's factorisation is the same computation, so the columns agree.
__global__ void __launch_bounds__(256) k_coarse_invert(Grid3 g, const float4* __restrict__ coef,
                                                       float* __restrict__ ainv, int pin) {
    // m x m with rows padded to m + 1 doubles (a column of 16 rows spans the
    // shared-memory banks instead of hitting one), then the y/x vector
    extern __shared__ double A[];
    const int m = g.nx * g.ny * g.nz, lda = m + 1;
    const int t = threadIdx.x, nt = blockDim.x;
    const int b = blockIdx.x;
    __shared__ int active[64];
    double* v = A + m * lda;  // right-hand side / solution
    for (int k = t; k < m * lda; k += nt) A[k] = 0.0;
    __syncthreads();
    if (t < m) {
        const int x = t % g.nx, y = (t / g.nx) % g.ny, z = t / (g.nx * g.ny);
        const float4 c = coef[t];
        double d = c.w;
        const int n3[3] = {g.nx, g.ny, g.nz}, p3[3] = {x, y, z};
        const float lowb[3] = {c.x, c.y, c.z};
        for (int a = 0; a < 3; a++) {
            const int stride = a == 0 ? 1 : (a == 1 ? g.nx : g.nx * g.ny);
            const int lm = wrap_or_neg(p3[a] - 1, n3[a], g.periodic & (1 << a));
            const int lp = wrap_or_neg(p3[a] + 1, n3[a], g.periodic & (1 << a));
            if (lm >= 0 && lowb[a] != 0.0f) {
                d += lowb[a];
                A[t * lda + (t + (lm - p3[a]) * stride)] -= lowb[a];
            }
            if (lp >= 0) {
                const int j = t + (lp - p3[a]) * stride;
                const float bh = (a == 0 ? coef[j].x : (a == 1 ? coef[j].y : coef[j].z));
                if (bh != 0.0f) {
                    d += bh;
                    A[t * lda + j] -= bh;
                }
            }
        }
        A[t * lda + t] += d;
        active[t] = d > 0.0 && t != pin;  // a pinned cell (mean-free gauge) is held at zero
    }
    __syncthreads();
    if (t < m && !active[t]) {
        for (int k = 0; k < m; k++) A[t * lda + k] = A[k * lda + t] = 0.0;
        A[t * lda + t] = 1.0;
    }
    __syncthreads();
    // Cholesky, lower triangle in place (a non-positive pivot is treated as
    // an empty row).  FP64 divisions and square roots are long dependent
    // sequences on this part, so each pivot takes one reciprocal square root
    // (rsq[j] = 1 / L_jj, an FP32 seed refined by two Newton-Raphson steps
    // r <- r (3 - a r^2) / 2 in FP64) and the column is scaled by it.
    __shared__ double rsq[64];
    const int tx = t & 15, ty = t >> 4;
    for (int j = 0; j < m; j++) {
        if (t == 0) {
            const double piv = A[j * lda + j];
            double r = 0.0;
            if (piv > 1e-30 && piv < 1e30) {
                r = (double)rsqrtf((float)piv);
                r = r * (1.5 - 0.5 * piv * r * r);
                r = r * (1.5 - 0.5 * piv * r * r);
            } else if (piv > 1e-300) {
                r = 1.0 / sqrt(piv);
            }
            A[j * lda + j] = piv * r;  // L_jj (0 for an empty row)
            rsq[j] = r;
        }
        __syncthreads();
        const double rj = rsq[j];
        for (int i = j + 1 + t; i < m; i += nt) A[i * lda + j] *= rj;
        __syncthreads();
        for (int i = j + 1 + ty; i < m; i += 16)
            for (int k = j + 1 + tx; k <= i; k += 16) A[i * lda + k] -= A[i * lda + j] * A[k * lda + j];
        __syncthreads();
    }
    // L y = e_b, then L^T x = y, column-oriented: thread i keeps v[i]; step j
    // finishes v[j] and updates the rows after it (before it, going back).
    if (t < m) v[t] = t == b ? 1.0 : 0.0;
    __syncthreads();
    for (int j = 0; j < m; j++) {
        const double yj = v[j] * rsq[j];
        __syncthreads();
        if (t == j) v[j] = yj;
        else if (t > j && t < m) v[t] -= A[t * lda + j] * yj;
        __syncthreads();
    }
    for (int j = m - 1; j >= 0; j--) {
        const double xj = v[j] * rsq[j];
        __syncthreads();
        if (t == j) v[j] = xj;
        else if (t < j) v[t] -= A[j * lda + t] * xj;
        __syncthreads();
    }
    __syncthreads();
    for (int i = t; i < m; i += nt)
        ainv[i * m + b] = (active[i] && active[b]) ? (float)v[i] : 0.0f;
}

// -------------------------------------------------- bottom sub-cycle
// The levels of at most 4096 cells in one block of 1024 threads: the whole
// sub-V-cycle below level B (pre-smoothing and restriction down, the exact
// coarsest solve, prolongation and post-smoothing up) runs out of shared
// memory with a barrier between steps instead of a launch per step.  Each
// cell does the operations of k_smooth / k_restrict / k_prolong /
// k_coarse_solve on the same level fields, with the diagonal summed once per
// launch and the smoother's division by the fast reciprocal (a fixed factor
// per cell, so the sub-cycle stays a fixed symmetric operator).
constexpr int BOTTOM_THREADS = 1024;

// Cell lists of the bottom sub-cycle: per level the red cells, then the
// black ones, each colour in index order.  On a grid without periodic axes a
// list entry is a flat word: the cell index (bits 0-12), which of its six
// neighbours exist (bits 13-18: x-, x+, y-, y+, z-, z+) and its parent cell
// on the next level (bits 19-31), so the loops decode no coordinates and
// test no wrap-around.  With a periodic axis an entry holds the packed
// coordinates x | y << 10 | z << 20 and the loops take the wrap-aware path.
constexpr unsigned BW_XM = 1u << 13, BW_XP = 1u << 14, BW_YM = 1u << 15, BW_YP = 1u << 16, BW_ZM = 1u << 17,
                   BW_ZP = 1u << 18;
__device__ __forceinline__ int bw_index(unsigned w) { return (int)(w & 0x1fffu); }
// A level's records in shared memory, one array per lane (beta_x, beta_y,
// beta_z of the low faces, diagonal): the cells of one colour sit two apart,
// so a float4 record per cell made each neighbour-face load an eight-way bank
// conflict; with separate arrays it is two-way.
struct RecSoA {
    float *bx, *by, *bz, *d;
    __device__ __forceinline__ RecSoA(float* base, int n) : bx(base), by(base + n), bz(base + 2 * n), d(base + 3 * n) {}
};
__device__ __forceinline__ int bw_parent(unsigned w) { return (int)(w >> 19); }

// Exclusive prefix sum of one count per thread over the block (blockDim.x a
// multiple of 32, at most 1024).
__device__ int block_exclusive_scan(int v, int* warp_tot) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int s = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += u;
    }
    if (lane == 31) warp_tot[wid] = s;
    __syncthreads();
    if (wid == 0) {
        int w = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += u;
        }
        warp_tot[lane] = w;  // inclusive totals of warps 0 .. lane
    }
    __syncthreads();
    const int r = (wid ? warp_tot[wid - 1] : 0) + s - v;
    __syncthreads();  // warp_tot is reused by the next call
    return r;
}

// The shared-memory image of the bottom sub-cycle that depends only on the
// coefficients, built once per coefficient set: per level the records with
// the diagonal in place of the reaction (k_smooth's sum order) and the cell
// list; then the coarsest inverse.  Every launch of k_bottom_vcycle copies it
// in with 16-byte cp.async.
template <int CK>
__global__ void __launch_bounds__(BOTTOM_THREADS) k_bottom_image(BottomPlan B, float4* __restrict__ img) {
    extern __shared__ float4 bsm4[];
    float* bsm = reinterpret_cast<float*>(bsm4);
    const int t = threadIdx.x, nt = blockDim.x;
    auto nb = [](int c, int n, bool per) { return wrap_or_neg(c, n, per); };
    __shared__ int warp_tot[32];
    for (int l = 0; l < B.nl; l++) {
        const BottomLevel& L = B.lv[l];
        const Grid3& g = L.g;
        const RecSoA c(bsm + 4 * L.coff, L.n);
        unsigned* cells = reinterpret_cast<unsigned*>(bsm + L.xoff);
        for (int i = t; i < L.n; i += nt) {
            const float4 v = ldc<CK>(L.coef, i);
            c.bx[i] = v.x;
            c.by[i] = v.y;
            c.bz[i] = v.z;
            c.d[i] = v.w;
        }
        // thread t lists the cells of one contiguous chunk; a scan of the red
        // counts gives each cell its place in the colour-ordered list
        const int chunk = (L.n + nt - 1) / nt;
        const int i0 = min(L.n, t * chunk), i1 = min(L.n, i0 + chunk);
        int red = 0;
        for (int i = i0; i < i1; i++) {
            const int x = i % g.nx, y = (i / g.nx) % g.ny, z = i / (g.nx * g.ny);
            red += ((x + y + z) & 1) == 0;
        }
        int rk = block_exclusive_scan(red, warp_tot);  // red cells before i0
        const bool flat = g.periodic == 0;
        const Grid3 gc = l + 1 < B.nl ? B.lv[l + 1].g : g;
        for (int i = i0; i < i1; i++) {
            const int x = i % g.nx, y = (i / g.nx) % g.ny, z = i / (g.nx * g.ny);
            unsigned w;
            if (flat) {
                w = (unsigned)i;
                if (x > 0) w |= BW_XM;
                if (x + 1 < g.nx) w |= BW_XP;
                if (y > 0) w |= BW_YM;
                if (y + 1 < g.ny) w |= BW_YP;
                if (z > 0) w |= BW_ZM;
                if (z + 1 < g.nz) w |= BW_ZP;
                if (l + 1 < B.nl) w |= (unsigned)((x >> 1) + gc.nx * ((y >> 1) + gc.ny * (z >> 1))) << 19;
            } else {
                w = (unsigned)(x | (y << 10) | (z << 20));
            }
            if (((x + y + z) & 1) == 0) cells[rk++] = w;
            else cells[L.nred + (i - rk)] = w;  // i - rk black cells precede i
        }
    }
    __syncthreads();
    // the diagonal replaces the reaction in each record (k_smooth's sum order)
    for (int l = 0; l < B.nl; l++) {
        const BottomLevel& L = B.lv[l];
        const Grid3& g = L.g;
        const RecSoA c(bsm + 4 * L.coff, L.n);
        float* dtmp = bsm + L.off + 2 * L.n;  // scratch until the cycle starts
        const bool px = g.periodic & 1, py = g.periodic & 2, pz = g.periodic & 4;
        for (int i = t; i < L.n; i += nt) {
            const int x = i % g.nx, y = (i / g.nx) % g.ny, z = i / (g.nx * g.ny);
            const int xp = nb(x + 1, g.nx, px), yp = nb(y + 1, g.ny, py), zp = nb(z + 1, g.nz, pz);
            const float bxh = xp >= 0 ? c.bx[i + (xp - x)] : 0.f;
            const float byh = yp >= 0 ? c.by[i + (yp - y) * g.nx] : 0.f;
            const float bzh = zp >= 0 ? c.bz[i + (zp - z) * g.nx * g.ny] : 0.f;
            dtmp[i] = ((c.bx[i] + bxh) + (c.by[i] + byh)) + ((c.bz[i] + bzh) + c.d[i]);
        }
    }
    __syncthreads();
    for (int l = 0; l < B.nl; l++) {
        const BottomLevel& L = B.lv[l];
        const RecSoA c(bsm + 4 * L.coff, L.n);
        const float* dtmp = bsm + L.off + 2 * L.n;
        for (int i = t; i < L.n; i += nt) c.d[i] = dtmp[i];
    }
    __syncthreads();
    for (int i = t; i < B.m * B.m; i += nt) bsm[B.aoff + i] = B.ainv[i];
    __syncthreads();
    for (int i = t; i < B.img_floats / 4; i += nt) img[i] = bsm4[i];
}

template <int CK, class VT>
__global__ void __launch_bounds__(BOTTOM_THREADS) k_bottom_vcycle(BottomPlan B, const Scalars* sc) {
    if (sc->converged) return;
    extern __shared__ float4 bsm4[];
    float* bsm = reinterpret_cast<float*>(bsm4);
    const int t = threadIdx.x, nt = blockDim.x;
    for (int i = t; i < B.img_floats / 4; i += nt) staged::cp_async16(bsm4 + i, B.img + i, true);
    staged::cp_commit();
    {
        const BottomLevel& L = B.lv[0];
        float* r = bsm + L.off;
        const VT* rg = reinterpret_cast<const VT*>(L.r);
        for (int i = t; i < L.n; i += nt) r[i] = to_f(rg[i]);
    }
    staged::cp_wait<0>();
    __syncthreads();
    auto nb = [](int c, int n, bool per) { return wrap_or_neg(c, n, per); };
    // sum of beta * e over the six neighbours (k_smooth order) and the
    // diagonal; wrap-aware, for levels with a periodic axis
    auto stencil = [&](const BottomLevel& L, const RecSoA& c, const float* e, int x, int y, int z, int i, float acc,
                       float* d) {
        const Grid3& g = L.g;
        const bool px = g.periodic & 1, py = g.periodic & 2, pz = g.periodic & 4;
        const int sy = g.nx, sz = g.nx * g.ny;
        const int xm = nb(x - 1, g.nx, px), xp = nb(x + 1, g.nx, px);
        const int ym = nb(y - 1, g.ny, py), yp = nb(y + 1, g.ny, py);
        const int zm = nb(z - 1, g.nz, pz), zp = nb(z + 1, g.nz, pz);
        const float bxh = xp >= 0 ? c.bx[i + (xp - x)] : 0.f;
        const float byh = yp >= 0 ? c.by[i + (yp - y) * sy] : 0.f;
        const float bzh = zp >= 0 ? c.bz[i + (zp - z) * sz] : 0.f;
        *d = c.d[i];
        acc = fmaf(c.bx[i], xm >= 0 ? e[i + (xm - x)] : 0.f, acc);
        acc = fmaf(bxh, xp >= 0 ? e[i + (xp - x)] : 0.f, acc);
        acc = fmaf(c.by[i], ym >= 0 ? e[i + (ym - y) * sy] : 0.f, acc);
        acc = fmaf(byh, yp >= 0 ? e[i + (yp - y) * sy] : 0.f, acc);
        acc = fmaf(c.bz[i], zm >= 0 ? e[i + (zm - z) * sz] : 0.f, acc);
        acc = fmaf(bzh, zp >= 0 ? e[i + (zp - z) * sz] : 0.f, acc);
        return acc;
    };
    // the same sums for a flat list word: fixed strides, neighbour bits
    auto stencil_flat = [&](const RecSoA& c, const float* e, unsigned w, int sy, int sz, float acc, float* d) {
        const int i = bw_index(w);
        const float bxh = (w & BW_XP) ? c.bx[i + 1] : 0.f;
        const float byh = (w & BW_YP) ? c.by[i + sy] : 0.f;
        const float bzh = (w & BW_ZP) ? c.bz[i + sz] : 0.f;
        *d = c.d[i];
        acc = fmaf(c.bx[i], (w & BW_XM) ? e[i - 1] : 0.f, acc);
        acc = fmaf(bxh, (w & BW_XP) ? e[i + 1] : 0.f, acc);
        acc = fmaf(c.by[i], (w & BW_YM) ? e[i - sy] : 0.f, acc);
        acc = fmaf(byh, (w & BW_YP) ? e[i + sy] : 0.f, acc);
        acc = fmaf(c.bz[i], (w & BW_ZM) ? e[i - sz] : 0.f, acc);
        acc = fmaf(bzh, (w & BW_ZP) ? e[i + sz] : 0.f, acc);
        return acc;
    };
    auto half_step = [&](int l, int color, bool zero) {
        const BottomLevel& L = B.lv[l];
        const Grid3& g = L.g;
        const RecSoA c(bsm + 4 * L.coff, L.n);
        const unsigned* cells = reinterpret_cast<const unsigned*>(bsm + L.xoff);
        const float* r = bsm + L.off;
        float* e = bsm + L.off + L.n;
        float* tmp = bsm + L.off + 2 * L.n;
        const bool flat = g.periodic == 0;
        if (zero) {  // from zero: red cells r / d, black cells 0
#pragma unroll 4
            for (int k = t; k < L.n; k += nt) {
                const unsigned cc = cells[k];
                int i;
                if (flat) {
                    i = bw_index(cc);
                } else {
                    const int x = cc & 1023, y = (cc >> 10) & 1023, z = cc >> 20;
                    i = x + g.nx * (y + g.ny * z);
                }
                float val = 0.f;
                if (k < L.nred) {
                    const float d = c.d[i];
                    if (d > 0.f) val = __fdividef(r[i], d);
                }
                e[i] = val;
            }
            __syncthreads();
            return;
        }
        const int k0 = color ? L.nred : 0, k1 = color ? L.n : L.nred;
        if (flat) {  // never odd: odd extents only matter on periodic axes
            const int sy = g.nx, sz = g.nx * g.ny;
#pragma unroll 2
            for (int k = k0 + t; k < k1; k += nt) {
                const unsigned w = cells[k];
                float d;
                const float acc = stencil_flat(c, e, w, sy, sz, r[bw_index(w)], &d);
                e[bw_index(w)] = d > 0.f ? __fdividef(acc, d) : 0.f;
            }
            __syncthreads();
            return;
        }
#pragma unroll 2
        for (int k = k0 + t; k < k1; k += nt) {
            const unsigned cc = cells[k];
            const int x = cc & 1023, y = (cc >> 10) & 1023, z = cc >> 20;
            const int i = x + g.nx * (y + g.ny * z);
            float d;
            const float acc = stencil(L, c, e, x, y, z, i, r[i], &d);
            const float val = d > 0.f ? __fdividef(acc, d) : 0.f;
            if (L.odd) tmp[i] = val;
            else e[i] = val;
        }
        __syncthreads();
        if (L.odd) {
            for (int k = k0 + t; k < k1; k += nt) {
                const unsigned cc = cells[k];
                const int x = cc & 1023, y = (cc >> 10) & 1023, z = cc >> 20;
                const int i = x + g.nx * (y + g.ny * z);
                e[i] = tmp[i];
            }
            __syncthreads();
        }
    };
    // Restriction right after the pre-smoothing half-steps.  Without odd
    // periodic extents the residual of a black cell is zero (its update
    // solved its equation) and that of a red cell is sum beta * e over its
    // black neighbours, so one pass forms those sums for the red cells and a
    // second adds each coarse cell's red children.
    auto restrict_to = [&](int l) {  // level l -> l+1
        const BottomLevel &F = B.lv[l], &C = B.lv[l + 1];
        const Grid3 &g = F.g, &gc = C.g;
        const RecSoA c(bsm + 4 * F.coff, F.n);
        const float* r = bsm + F.off;
        const float* e = bsm + F.off + F.n;
        float* rc = bsm + C.off;
        const unsigned* ccells = reinterpret_cast<const unsigned*>(bsm + C.xoff);
        if (!F.odd) {
            float* rs = bsm + F.off + 2 * F.n;
            const unsigned* cells = reinterpret_cast<const unsigned*>(bsm + F.xoff);
            if (g.periodic == 0) {
                const int sy = g.nx, sz = g.nx * g.ny;
#pragma unroll 2
                for (int k = t; k < F.nred; k += nt) {
                    const unsigned w = cells[k];
                    float d;
                    rs[bw_index(w)] = stencil_flat(c, e, w, sy, sz, 0.f, &d);
                }
            } else {
#pragma unroll 2
                for (int k = t; k < F.nred; k += nt) {
                    const unsigned cc = cells[k];
                    const int x = cc & 1023, y = (cc >> 10) & 1023, z = cc >> 20;
                    const int i = x + g.nx * (y + g.ny * z);
                    float d;
                    rs[i] = stencil(F, c, e, x, y, z, i, 0.f, &d);
                }
            }
            __syncthreads();
            for (int K = t; K < C.n; K += nt) {
                const int X = K % gc.nx, Y = (K / gc.nx) % gc.ny, Z = K / (gc.nx * gc.ny);
                float part = 0.f;
                for (int dz = 0; dz < 2; dz++)
                    for (int dy = 0; dy < 2; dy++)
                        for (int dx = 0; dx < 2; dx++) {
                            const int x = 2 * X + dx, y = 2 * Y + dy, z = 2 * Z + dz;
                            if (x >= g.nx || y >= g.ny || z >= g.nz || ((x + y + z) & 1)) continue;
                            part += rs[x + g.nx * (y + g.ny * z)];
                        }
                rc[K] = 0.25f * part;
            }
            __syncthreads();
            return;
        }
        for (int k = t; k < C.n; k += nt) {
            const unsigned cq = ccells[k];
            const int X = cq & 1023, Y = (cq >> 10) & 1023, Z = cq >> 20;
            float part = 0.f;
            for (int dz = 0; dz < 2; dz++)
                for (int dy = 0; dy < 2; dy++)
                    for (int dx = 0; dx < 2; dx++) {
                        const int x = 2 * X + dx, y = 2 * Y + dy, z = 2 * Z + dz;
                        if (x >= g.nx || y >= g.ny || z >= g.nz) continue;
                        const int i = x + g.nx * (y + g.ny * z);
                        float d;
                        const float nsum = stencil(F, c, e, x, y, z, i, 0.f, &d);
                        part += r[i] - (d * e[i] - nsum);
                    }
            rc[X + gc.nx * (Y + gc.ny * Z)] = 0.25f * part;
        }
        __syncthreads();
    };
    auto prolong_from = [&](int l) {  // level l+1 -> l
        const BottomLevel &F = B.lv[l], &C = B.lv[l + 1];
        const Grid3 &g = F.g, &gc = C.g;
        float* e = bsm + F.off + F.n;
        const float* ec = bsm + C.off + C.n;
        const unsigned* cells = reinterpret_cast<const unsigned*>(bsm + F.xoff);
        if (g.periodic == 0) {
            for (int k = t; k < F.n; k += nt) {
                const unsigned w = cells[k];
                const int i = bw_index(w);
                e[i] = fmaf(B.w, ec[bw_parent(w)], e[i]);
            }
        } else {
            for (int k = t; k < F.n; k += nt) {
                const unsigned cc = cells[k];
                const int x = cc & 1023, y = (cc >> 10) & 1023, z = cc >> 20;
                const int i = x + g.nx * (y + g.ny * z);
                e[i] = fmaf(B.w, ec[(x >> 1) + gc.nx * ((y >> 1) + gc.ny * (z >> 1))], e[i]);
            }
        }
        __syncthreads();
    };
    // The cycle program (host-generated): PRE / POST visits of a level,
    // the exact coarsest solve, and the second coarse visit of a W-cycle
    // level: save e and replace r by r - A e, then add the saved e back.
    for (int k = 0; k < B.nops; k++) {
        const int op = B.ops[k] >> 4, l = B.ops[k] & 15;
        if (op == BOP_PRE) {
            half_step(l, 0, true);
            half_step(l, 1, false);
            restrict_to(l);
        } else if (op == BOP_POST) {
            prolong_from(l);
            half_step(l, 1, false);
            half_step(l, 0, false);
        } else if (op == BOP_COARSE) {
            // e = ainv r, sixteen threads per row (m <= 64)
            const BottomLevel& K = B.lv[l];
            const float* r = bsm + K.off;
            float* e = bsm + K.off + K.n;
            const float* A = bsm + B.aoff;
            const int row = t >> 4, lane = t & 15;
            float sacc = 0.0f;
            if (row < B.m)
                for (int q = lane; q < B.m; q += 16) sacc = fmaf(A[row * B.m + q], r[q], sacc);
#pragma unroll
            for (int w = 8; w > 0; w >>= 1) sacc += __shfl_xor_sync(0xffffffffu, sacc, w, 16);
            if (row < B.m && lane == 0) e[row] = sacc;
            __syncthreads();
        } else if (op == BOP_SAVE_RESID) {
            const BottomLevel& L = B.lv[l];
            const Grid3& g = L.g;
            const RecSoA c(bsm + 4 * L.coff, L.n);
            const unsigned* cells = reinterpret_cast<const unsigned*>(bsm + L.xoff);
            float* r = bsm + L.off;
            const float* e = bsm + L.off + L.n;
            float* es = bsm + L.off + 3 * L.n;
            const bool flat = g.periodic == 0;
            const int sy = g.nx, sz = g.nx * g.ny;
            float rn[4];  // each thread's cells, at most 4096 / 1024
            int cnt = 0;
            for (int q = t; q < L.n; q += nt) {
                const unsigned cc = cells[q];
                float d, nsum;
                int i;
                if (flat) {
                    i = bw_index(cc);
                    nsum = stencil_flat(c, e, cc, sy, sz, 0.f, &d);
                } else {
                    const int x = cc & 1023, y = (cc >> 10) & 1023, z = cc >> 20;
                    i = x + g.nx * (y + g.ny * z);
                    nsum = stencil(L, c, e, x, y, z, i, 0.f, &d);
                }
                rn[cnt++] = r[i] - (d * e[i] - nsum);
            }
            __syncthreads();
            cnt = 0;
            for (int q = t; q < L.n; q += nt) {
                const unsigned cc = cells[q];
                int i;
                if (flat) {
                    i = bw_index(cc);
                } else {
                    const int x = cc & 1023, y = (cc >> 10) & 1023, z = cc >> 20;
                    i = x + g.nx * (y + g.ny * z);
                }
                r[i] = rn[cnt++];
                es[i] = e[i];
            }
            __syncthreads();
        } else if (op == BOP_ADD_SAVED) {
            const BottomLevel& L = B.lv[l];
            float* e = bsm + L.off + L.n;
            const float* es = bsm + L.off + 3 * L.n;
            for (int i = t; i < L.n; i += nt) e[i] += es[i];
            __syncthreads();
        }
    }
    {
        const BottomLevel& L = B.lv[0];
        const float* e = bsm + L.off + L.n;
        VT* eg = reinterpret_cast<VT*>(L.e);
        for (int i = t; i < L.n; i += nt) eg[i] = from_f<VT>(e[i]);
    }
}

// ------------------------------------------------------------- host side
template <int CK, class VT>
static void enqueue_smooth(const MGPlan& P, int l, int color, bool zero, cudaStream_t s) {
    const MGLevel& L = P.lv[l];
    const void* coef = P.precision == 0 ? (const void*)L.coef32 : L.coef_lo;
    if (l == 0 && P.staged) {
        launch_smooth_staged(CK, L.L, coef, (const float*)L.r, (float*)L.e, (float*)L.tmp, color, zero,
                             L.odd_periodic, P.sc, s);
        if (!zero && L.odd_periodic)
            k_copy_color<float><<<L.L.grid, L.L.block, 0, s>>>(L.L.g, (const float*)L.tmp, (float*)L.e, color, P.sc);
        return;
    }
    if (l == 0) {
        const float* r = (const float*)L.r;
        float* e = (float*)L.e;
        if (zero) k_smooth<CK, float, true, true, false><<<L.L.grid, L.L.block, 0, s>>>(L.L.g, coef, r, e, e, color, P.sc);
        else if (!L.odd_periodic)
            k_smooth<CK, float, true, false, false><<<L.L.grid, L.L.block, 0, s>>>(L.L.g, coef, r, e, e, color, P.sc);
        else {
            float* t = (float*)L.tmp;
            k_smooth<CK, float, true, false, true><<<L.L.grid, L.L.block, 0, s>>>(L.L.g, coef, r, e, t, color, P.sc);
            k_copy_color<float><<<L.L.grid, L.L.block, 0, s>>>(L.L.g, t, e, color, P.sc);
        }
    } else {
        const VT* r = (const VT*)L.r;
        VT* e = (VT*)L.e;
        if (zero) k_smooth<CK, VT, false, true, false><<<L.L.grid, L.L.block, 0, s>>>(L.L.g, coef, r, e, e, color, P.sc);
        else if (!L.odd_periodic)
            k_smooth<CK, VT, false, false, false><<<L.L.grid, L.L.block, 0, s>>>(L.L.g, coef, r, e, e, color, P.sc);
        else {
            VT* t = (VT*)L.tmp;
            k_smooth<CK, VT, false, false, true><<<L.L.grid, L.L.block, 0, s>>>(L.L.g, coef, r, e, t, color, P.sc);
            k_copy_color<VT><<<L.L.grid, L.L.block, 0, s>>>(L.L.g, t, e, color, P.sc);
        }
    }
}

// Levels l0 .. nlevels-1 of the V-cycle: pre-smoothing and restriction down
// from l0, the exact coarsest solve, prolongation and post-smoothing back up
// to l0.  The caller prolongs level l0's correction further up.
template <int CK, class VT>
static void vcycle_impl(const MGPlan& P, int l0, cudaStream_t s) {
    const int nl = P.nlevels;
    // levels from P.bottom_from down run in the bottom sub-cycle kernel
    const int lb = (P.bottom_from > 0 && P.bottom_from >= l0) ? P.bottom_from : nl;
    for (int l = l0; l + 1 < nl && l < lb; l++) {
        enqueue_smooth<CK, VT>(P, l, 0, true, s);
        enqueue_smooth<CK, VT>(P, l, 1, false, s);
        const MGLevel &F = P.lv[l], &C = P.lv[l + 1];
        const void* coef = P.precision == 0 ? (const void*)F.coef32 : F.coef_lo;
        if (l == 0 && P.staged)
            launch_restrict_staged(CK, F.L, C.L.g, coef, (const float*)F.r, (const float*)F.e, C.r, P.sc, s);
        else if (l == 0)
            k_restrict<CK, float, true, VT><<<F.L.grid, F.L.block, 0, s>>>(F.L.g, C.L.g, coef, (const float*)F.r,
                                                                           (const float*)F.e, (VT*)C.r, P.sc);
        else
            k_restrict<CK, VT, false, VT><<<F.L.grid, F.L.block, 0, s>>>(F.L.g, C.L.g, coef, (const VT*)F.r,
                                                                         (const VT*)F.e, (VT*)C.r, P.sc);
    }
    if (lb < nl) {
        k_bottom_vcycle<CK, VT><<<1, BOTTOM_THREADS, P.bottom_smem, s>>>(P.bottom, P.sc);
    } else {
        const MGLevel& K = P.lv[nl - 1];
        if (nl == 1) k_coarse_solve<float, true><<<1, 64, 0, s>>>(P.m, P.ainv, (const float*)K.r, (float*)K.e, P.sc);
        else k_coarse_solve<VT, false><<<1, 64, 0, s>>>(P.m, P.ainv, (const VT*)K.r, (VT*)K.e, P.sc);
    }
    for (int l = std::min(nl - 2, lb - 1); l >= l0; l--) {
        const MGLevel &F = P.lv[l], &C = P.lv[l + 1];
        if (l == 0)
            k_prolong<float, VT><<<F.L.grid, F.L.block, 0, s>>>(F.L.g, C.L.g, (float*)F.e, (const VT*)C.e, P.prolong, P.sc);
        else
            k_prolong<VT, VT><<<F.L.grid, F.L.block, 0, s>>>(F.L.g, C.L.g, (VT*)F.e, (const VT*)C.e, P.prolong, P.sc);
        enqueue_smooth<CK, VT>(P, l, 1, false, s);
        enqueue_smooth<CK, VT>(P, l, 0, false, s);
    }
}

void mg_vcycle_from(const MGPlan& P, int l0, cudaStream_t s) {
    if (P.precision == 1) vcycle_impl<1, __half>(P, l0, s);
    else if (P.precision == 2) vcycle_impl<2, __nv_bfloat16>(P, l0, s);
    else vcycle_impl<0, float>(P, l0, s);
}

void mg_vcycle(const MGPlan& P, cudaStream_t s) { mg_vcycle_from(P, 0, s); }

// One launch of the bottom sub-cycle on its current right-hand side, for
// measurement.
void mg_bottom_cycle(const MGPlan& P, cudaStream_t s) {
    if (P.bottom_from <= 0) return;
    if (P.precision == 1) k_bottom_vcycle<1, __half><<<1, BOTTOM_THREADS, P.bottom_smem, s>>>(P.bottom, P.sc);
    else if (P.precision == 2)
        k_bottom_vcycle<2, __nv_bfloat16><<<1, BOTTOM_THREADS, P.bottom_smem, s>>>(P.bottom, P.sc);
    else k_bottom_vcycle<0, float><<<1, BOTTOM_THREADS, P.bottom_smem, s>>>(P.bottom, P.sc);
}

template <int CK, class VT>
static void fine_restrict_impl(const MGPlan& P, cudaStream_t s) {
    const MGLevel &F = P.lv[0], &C = P.lv[1];
    const void* coef = P.precision == 0 ? (const void*)F.coef32 : F.coef_lo;
    if (P.staged) {
        launch_restrict_staged(CK, F.L, C.L.g, coef, (const float*)F.r, (const float*)F.e, C.r, P.sc, s);
        return;
    }
    k_restrict<CK, float, true, VT><<<F.L.grid, F.L.block, 0, s>>>(F.L.g, C.L.g, coef, (const float*)F.r,
                                                                   (const float*)F.e, (VT*)C.r, P.sc);
}
template <class VT>
static void fine_prolong_impl(const MGPlan& P, cudaStream_t s) {
    const MGLevel &F = P.lv[0], &C = P.lv[1];
    k_prolong<float, VT><<<F.L.grid, F.L.block, 0, s>>>(F.L.g, C.L.g, (float*)F.e, (const VT*)C.e, P.prolong, P.sc);
}
void mg_fine_smooth(const MGPlan& P, int color, cudaStream_t s) {
    if (P.precision == 1) enqueue_smooth<1, __half>(P, 0, color, false, s);
    else if (P.precision == 2) enqueue_smooth<2, __nv_bfloat16>(P, 0, color, false, s);
    else enqueue_smooth<0, float>(P, 0, color, false, s);
}
void mg_fine_restrict(const MGPlan& P, cudaStream_t s) {
    if (P.nlevels < 2) return;
    if (P.precision == 1) fine_restrict_impl<1, __half>(P, s);
    else if (P.precision == 2) fine_restrict_impl<2, __nv_bfloat16>(P, s);
    else fine_restrict_impl<0, float>(P, s);
}
void mg_fine_prolong(const MGPlan& P, cudaStream_t s) {
    if (P.nlevels < 2) return;
    if (P.precision == 1) fine_prolong_impl<__half>(P, s);
    else if (P.precision == 2) fine_prolong_impl<__nv_bfloat16>(P, s);
    else fine_prolong_impl<float>(P, s);
}

void mg_build(const MGPlan& P, cudaStream_t s) {
    for (int l = 1; l < P.nlevels; l++) {
        const MGLevel &F = P.lv[l - 1], &C = P.lv[l];
        if (P.precision == 1)
            k_mg_build<1><<<C.L.grid, C.L.block, 0, s>>>(F.L.g, C.L.g, F.coef32, C.coef32, C.coef_lo);
        else if (P.precision == 2)
            k_mg_build<2><<<C.L.grid, C.L.block, 0, s>>>(F.L.g, C.L.g, F.coef32, C.coef32, C.coef_lo);
        else
            k_mg_build<0><<<C.L.grid, C.L.block, 0, s>>>(F.L.g, C.L.g, F.coef32, C.coef32, nullptr);
    }
    const MGLevel& K = P.lv[P.nlevels - 1];
    const size_t smem = ((size_t)P.m * (P.m + 1) + P.m) * sizeof(double);
    k_coarse_invert<<<P.m, 256, smem, s>>>(K.L.g, K.coef32, P.ainv, P.pin_coarse);
    if (P.bottom_from > 0 && P.bottom_img) {
        if (P.precision == 1) k_bottom_image<1><<<1, BOTTOM_THREADS, P.bottom_smem, s>>>(P.bottom, P.bottom_img);
        else if (P.precision == 2) k_bottom_image<2><<<1, BOTTOM_THREADS, P.bottom_smem, s>>>(P.bottom, P.bottom_img);
        else k_bottom_image<0><<<1, BOTTOM_THREADS, P.bottom_smem, s>>>(P.bottom, P.bottom_img);
    }
}

cudaError_t mg_prepare_attributes() {
    cudaError_t e = cudaFuncSetAttribute(k_coarse_invert, cudaFuncAttributeMaxDynamicSharedMemorySize, (64 * 65 + 64) * 8);
    const int bmax = (int)BOTTOM_SMEM_MAX;
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_bottom_vcycle<0, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, bmax);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_bottom_vcycle<1, __half>, cudaFuncAttributeMaxDynamicSharedMemorySize, bmax);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_bottom_vcycle<2, __nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize, bmax);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_bottom_image<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, bmax);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_bottom_image<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, bmax);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_bottom_image<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, bmax);
    return e;
}

// The bottom sub-cycle from the first level of at most 4096 cells (level >= 1),
// if its levels fit the shared-memory budget.
void mg_plan_bottom(MGPlan& P) {
    P.bottom_from = 0;
    P.bottom_smem = 0;
    // Two coarse visits (a W-cycle step) on the first coarse level of at most
    // 32^3 cells: it costs little next to the fine level and cuts the CG
    // iterations by about a quarter on the jet workloads; deeper levels keep
    // V-cycles (their extra visits cost more barrier steps than they save).
    // The second visit, e1 + B (r - A e1), is positive definite only while
    // the inner cycle B converges on that level, which the weight-2 coarse
    // correction does not guarantee; the solver falls back to V-cycles
    // (w_disabled) when CG breaks down.
    P.w_from = P.w_to = 0;
    for (int l = 1; l + 1 < P.nlevels && !P.w_disabled; l++)
        if (P.lv[l].L.g.n() <= 32768) {
            P.w_from = P.w_to = l;  // two visits on that one level; V-cycles below it
            break;
        }
    int lb = -1;
    for (int l = 1; l < P.nlevels; l++)
        if (P.lv[l].L.g.n() <= 4096) {
            lb = l;
            break;
        }
    if (lb < 0 || P.nlevels - lb > 8 || P.m > BOTTOM_THREADS / 16) return;
    BottomPlan& B = P.bottom;
    B.nl = P.nlevels - lb;
    // Shared memory: the image (records of every level as float4s, the
    // cell lists, the coarsest inverse), then per level r, e, scratch and
    // saved e (floats).
    size_t f4 = 0;
    for (int k = 0; k < B.nl; k++) f4 += (size_t)P.lv[lb + k].L.g.n();
    size_t fl = 4 * f4;
    for (int k = 0; k < B.nl; k++) {
        B.lv[k].xoff = (int)fl;
        fl += (size_t)P.lv[lb + k].L.g.n();  // cell list (ints)
    }
    B.aoff = (int)fl;
    fl += (size_t)P.m * P.m;
    fl = (fl + 3) & ~(size_t)3;
    B.img_floats = (int)fl;
    for (int k = 0; k < B.nl; k++) {
        const MGLevel& L = P.lv[lb + k];
        BottomLevel& b = B.lv[k];
        b.g = L.L.g;
        b.n = (int)L.L.g.n();
        b.coef = P.precision == 0 ? (const void*)L.coef32 : L.coef_lo;
        b.r = L.r;
        b.e = L.e;
        b.odd = L.odd_periodic;
        b.coff = k == 0 ? 0 : B.lv[k - 1].coff + B.lv[k - 1].n;
        b.off = (int)fl;
        fl += 4 * (size_t)b.n;  // r, e, scratch, saved e
        int nred = 0;
        for (int z = 0; z < b.g.nz; z++)
            for (int y = 0; y < b.g.ny; y++)
                for (int x = 0; x < b.g.nx; x++) nred += ((x + y + z) & 1) == 0;
        b.nred = nred;
    }
    for (int k = 0; k < B.nl; k++)
        if (B.lv[k].g.nx > 1023 || B.lv[k].g.ny > 1023 || B.lv[k].g.nz > 1023) return;
    B.ainv = P.ainv;
    B.m = P.m;
    B.w = P.prolong;
    B.img = P.bottom_img;
    const size_t bytes = fl * sizeof(float);
    if (bytes > BOTTOM_SMEM_MAX) return;
    // the cycle program: level k's coarse correction takes two visits when
    // level lb + k is a W-cycle level (the program is cut back to V visits
    // if it would not fit)
    for (int attempt = 0; attempt < 2; attempt++) {
        const bool w_ok = attempt == 0;
        B.nops = 0;
        bool fits = true;
        auto emit = [&](int op, int l) {
            if (B.nops < BOTTOM_MAX_OPS) B.ops[B.nops++] = (unsigned char)((op << 4) | l);
            else fits = false;
        };
        std::function<void(int)> solve_level = [&](int k) {
            if (k == B.nl - 1) {
                emit(BOP_COARSE, k);
                return;
            }
            const bool w = w_ok && P.w_from > 0 && lb + k >= P.w_from && lb + k <= P.w_to;
            emit(BOP_PRE, k);
            solve_level(k + 1);
            emit(BOP_POST, k);
            if (w) {
                emit(BOP_SAVE_RESID, k);
                emit(BOP_PRE, k);
                solve_level(k + 1);
                emit(BOP_POST, k);
                emit(BOP_ADD_SAVED, k);
            }
        };
        solve_level(0);
        if (fits) break;
    }
    P.bottom_from = lb;
    P.bottom_smem = bytes;
}

}  // namespace mhdproj
