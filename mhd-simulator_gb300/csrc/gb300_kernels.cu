// gb300_kernels.cu -- fine-level kernels of the GB300 projection.
//
// Layout in HBM (x-fastest, cell i = x + nx*(y + ny*z)):
//   coef  float4[n]  (beta_x, beta_y, beta_z of the low faces, reaction)
//   cls   uint8[n]   0 solid, 1 active, 2 pinned gauge cell
//   b64, phi64 double[n]; r, z, p, q, e float[n]
//   faces u[(nx+1) ny nz], v[nx (ny+1) nz], w[nx ny (nz+1)]
// Every kernel walks 32x8 (x, y) tiles over a run of z, so warps read 128-byte
// rows and neighbouring z-planes are reused from L2.  Reductions are FP64:
// warp shuffles, one partial per block, and a deterministic fixed-order sum
// in the last block to finish, which also updates the CG scalars.
#include "kernels.h"

namespace mhdproj {

#define TILE_BEGIN(G)                                      \
    const int x = blockIdx.x * TX + threadIdx.x;           \
    const int y = blockIdx.y * TY + threadIdx.y;           \
    const bool in_xy = x < (G).nx && y < (G).ny;           \
    const int z0 = blockIdx.z * (G).zper;                  \
    const int z1 = min((G).nz, z0 + (G).zper);             \
    for (int z = z0; z < z1; z++)

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
__global__ void k_init_scalars(Scalars* sc, double tol2, double abs_floor, double inner_floor2) {
    sc->tol2 = tol2;
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

// Power-of-two scale that brings the RMS residual near 1/16, so FP16 level
// fields keep their values inside the normal range.
__device__ __forceinline__ void set_sigma_from(Scalars* sc, double rr, long long n_active) {
    double rms = n_active > 0 ? sqrt(rr / (double)n_active) : 0.0;
    if (rms > 0.0 && isfinite(rms)) {
        int ex;
        frexp(rms, &ex);
        double s = ldexp(1.0, -ex - 4);
        sc->sigma = (float)s;
        sc->inv_sigma = (float)(1.0 / s);
    } else {
        sc->sigma = 1.0f;
        sc->inv_sigma = 1.0f;
    }
}

// ------------------------------------------------------- coefficients
__global__ void __launch_bounds__(TILE_THREADS) k_coefficients(Grid3 g, int outlet, const float* __restrict__ alpha,
                                                               const uint8_t* __restrict__ cls, float rho_l,
                                                               float rho_air, float4* __restrict__ coef,
                                                               void* __restrict__ lo, int lo_kind,
                                                               float* __restrict__ gtop) {
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        const Nbr nb = neighbours(g, x, y, z);
        float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
        const uint8_t ci = cls[i];
        if (ci == 1) {
            const float ai = alpha[i];
            if (nb.xm >= 0 && cls[nb.xm] == 1) c.x = beta_of(alpha[nb.xm], ai, rho_l, rho_air);
            if (nb.ym >= 0 && cls[nb.ym] == 1) c.y = beta_of(alpha[nb.ym], ai, rho_l, rho_air);
            if (nb.zm >= 0 && cls[nb.zm] == 1) c.z = beta_of(alpha[nb.zm], ai, rho_l, rho_air);
            float r = 0.0f;
            const int order[6] = {nb.xm, nb.xp, nb.ym, nb.yp, nb.zm, nb.zp};
#pragma unroll
            for (int k = 0; k < 6; k++) {
                const int j = order[k];
                if (j >= 0 && cls[j] == 2) r = __fadd_rn(r, beta_of(ai, alpha[j], rho_l, rho_air));
            }
            if (outlet && z == g.nz - 1) {
                const float gt = outlet_conductance(ai, rho_l, rho_air);
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
// b = -h * sum over open faces of (u_high - u_low), FP64; ||b||^2.
__global__ void __launch_bounds__(TILE_THREADS) k_rhs(Grid3 g, int outlet, float h, const uint8_t* __restrict__ cls,
                                                      const float* __restrict__ u, const float* __restrict__ v,
                                                      const float* __restrict__ w, double* __restrict__ b,
                                                      Scalars* sc, double* partials, int nblocks) {
    __shared__ double sh[8 * 1];
    double acc[1] = {0.0};
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        double bi = 0.0;
        if (cls[i] == 1) {
            const Nbr nb = neighbours(g, x, y, z);
            double sum = 0.0;
            {
                const int hx = (x + 1 == nx && (g.periodic & 1)) ? 0 : x + 1;
                const double lo = (nb.xm >= 0 && cls[nb.xm] != 0) ? (double)u[x + (nx + 1) * (y + ny * z)] : 0.0;
                const double hi = (nb.xp >= 0 && cls[nb.xp] != 0) ? (double)u[hx + (nx + 1) * (y + ny * z)] : 0.0;
                sum += hi - lo;
            }
            {
                const int hy = (y + 1 == ny && (g.periodic & 2)) ? 0 : y + 1;
                const double lo = (nb.ym >= 0 && cls[nb.ym] != 0) ? (double)v[x + nx * (y + (ny + 1) * z)] : 0.0;
                const double hi = (nb.yp >= 0 && cls[nb.yp] != 0) ? (double)v[x + nx * (hy + (ny + 1) * z)] : 0.0;
                sum += hi - lo;
            }
            {
                const int hz = (z + 1 == nz && (g.periodic & 4)) ? 0 : z + 1;
                const double lo = (nb.zm >= 0 && cls[nb.zm] != 0) ? (double)w[x + nx * (y + ny * z)] : 0.0;
                const bool hopen = (nb.zp >= 0 && cls[nb.zp] != 0) || (outlet && z + 1 == nz);
                const double hi = hopen ? (double)w[x + nx * (y + ny * hz)] : 0.0;
                sum += hi - lo;
            }
            bi = -(double)h * sum;
        }
        b[i] = bi;
        acc[0] += bi * bi;
    }
    block_sum<1>(acc, sh);
    if (store_partials_is_last<1>(acc, partials, nblocks, &sc->ticket[0])) {
        double tot[1];
        finish_partials<1>(tot, partials, nblocks, sh, &sc->ticket[0]);
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            sc->bb = tot[0];
            if (!isfinite(tot[0])) sc->nonfinite = 1;
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
// r = b - A x in FP64 (x FP64), stored FP32 for the inner solve; e = 0.
__global__ void __launch_bounds__(TILE_THREADS) k_residual64(Grid3 g, const float4* __restrict__ coef,
                                                             const double* __restrict__ b,
                                                             const double* __restrict__ x64, float* __restrict__ r,
                                                             float* __restrict__ e, Scalars* sc, double* partials,
                                                             int nblocks, long long n_active) {
    __shared__ double sh[8 * 1];
    double acc[1] = {0.0};
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        const Nbr nb = neighbours(g, x, y, z);
        const double ri = b[i] - apply_cell<double>(g, coef, x64, i, nb);
        r[i] = (float)ri;
        e[i] = 0.0f;
        acc[0] += ri * ri;
    }
    block_sum<1>(acc, sh);
    if (store_partials_is_last<1>(acc, partials, nblocks, &sc->ticket[1])) {
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
        }
    }
}

// --------------------------------------------------------- CG kernels
__global__ void __launch_bounds__(TILE_THREADS) k_spmv_pq(Grid3 g, const float4* __restrict__ coef,
                                                          const float* __restrict__ p, float* __restrict__ q,
                                                          Scalars* sc, double* partials, int nblocks) {
    if (sc->converged) return;
    __shared__ double sh[8 * 1];
    double acc[1] = {0.0};
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        const Nbr nb = neighbours(g, x, y, z);
        const float qi = apply_cell<float>(g, coef, p, i, nb);
        q[i] = qi;
        acc[0] += (double)p[i] * (double)qi;
    }
    block_sum<1>(acc, sh);
    if (store_partials_is_last<1>(acc, partials, nblocks, &sc->ticket[2])) {
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

__global__ void __launch_bounds__(TILE_THREADS) k_update(Grid3 g, float* __restrict__ e, float* __restrict__ r,
                                                         const float* __restrict__ p, const float* __restrict__ q,
                                                         Scalars* sc, double* partials, int nblocks,
                                                         long long n_active) {
    if (sc->converged) return;
    __shared__ double sh[8 * 1];
    double acc[1] = {0.0};
    const float a = sc->alpha_f;
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        e[i] = fmaf(a, p[i], e[i]);
        const float ri = fmaf(-a, q[i], r[i]);
        r[i] = ri;
        acc[0] += (double)ri * (double)ri;
    }
    block_sum<1>(acc, sh);
    if (store_partials_is_last<1>(acc, partials, nblocks, &sc->ticket[3])) {
        double tot[1];
        finish_partials<1>(tot, partials, nblocks, sh, &sc->ticket[3]);
        if (threadIdx.x == 0 && threadIdx.y == 0) {
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
__global__ void __launch_bounds__(TILE_THREADS) k_dot_rz(Grid3 g, const float* __restrict__ r,
                                                         const float* __restrict__ zv, float* __restrict__ p, int init,
                                                         Scalars* sc, double* partials, int nblocks) {
    if (sc->converged) return;
    __shared__ double sh[8 * 1];
    double acc[1] = {0.0};
    const float is = sc->inv_sigma;
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        const float zi = zv[i] * is;
        if (init) p[i] = zi;
        acc[0] += (double)r[i] * (double)zi;
    }
    block_sum<1>(acc, sh);
    if (store_partials_is_last<1>(acc, partials, nblocks, &sc->ticket[4])) {
        double tot[1];
        finish_partials<1>(tot, partials, nblocks, sh, &sc->ticket[4]);
        if (threadIdx.x == 0 && threadIdx.y == 0) {
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

__global__ void __launch_bounds__(TILE_THREADS) k_search(Grid3 g, const float* __restrict__ zv, float* __restrict__ p,
                                                         const Scalars* sc) {
    if (sc->converged) return;
    const float is = sc->inv_sigma, bt = sc->beta_f;
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        p[i] = fmaf(bt, p[i], zv[i] * is);
    }
}

__global__ void __launch_bounds__(TILE_THREADS) k_accumulate(Grid3 g, double* __restrict__ x64,
                                                             const float* __restrict__ e) {
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        x64[i] += (double)e[i];
    }
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
// conductance against p = 0 on the face, closed faces are 0.  Each thread
// owns the low faces of its cell; the thread at index 0 of a periodic axis
// also writes the duplicate last face, the thread at the high end of a closed
// axis writes that wall face.
__global__ void __launch_bounds__(TILE_THREADS) k_correct(Grid3 g, int outlet, float h, float rho_l, float rho_air,
                                                          double p_scale, const uint8_t* __restrict__ cls,
                                                          const float* __restrict__ alpha,
                                                          const float* __restrict__ gtop,
                                                          const double* __restrict__ phi,
                                                          const float* __restrict__ us, const float* __restrict__ vs,
                                                          const float* __restrict__ ws, float* __restrict__ uo,
                                                          float* __restrict__ vo, float* __restrict__ wo,
                                                          float* __restrict__ po) {
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const double hd = (double)h;
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        const Nbr nb = neighbours(g, x, y, z);
        const uint8_t ci = cls[i];
        const double pi = phi[i];
        // x low face
        {
            const int f = x + (nx + 1) * (y + ny * z);
            float out = 0.0f;
            if (nb.xm >= 0 && ci != 0 && cls[nb.xm] != 0) {
                const float bt = beta_of(alpha[nb.xm], alpha[i], rho_l, rho_air);
                out = (float)((double)us[f] - (double)bt * (pi - phi[nb.xm]) / hd);
            }
            uo[f] = out;
            if (x == 0 && (g.periodic & 1)) uo[nx + (nx + 1) * (y + ny * z)] = out;
            if (x == nx - 1 && !(g.periodic & 1)) uo[nx + (nx + 1) * (y + ny * z)] = 0.0f;
        }
        {
            const int f = x + nx * (y + (ny + 1) * z);
            float out = 0.0f;
            if (nb.ym >= 0 && ci != 0 && cls[nb.ym] != 0) {
                const float bt = beta_of(alpha[nb.ym], alpha[i], rho_l, rho_air);
                out = (float)((double)vs[f] - (double)bt * (pi - phi[nb.ym]) / hd);
            }
            vo[f] = out;
            if (y == 0 && (g.periodic & 2)) vo[x + nx * (ny + (ny + 1) * z)] = out;
            if (y == ny - 1 && !(g.periodic & 2)) vo[x + nx * (ny + (ny + 1) * z)] = 0.0f;
        }
        {
            const int f = x + nx * (y + ny * z);
            float out = 0.0f;
            if (nb.zm >= 0 && ci != 0 && cls[nb.zm] != 0) {
                const float bt = beta_of(alpha[nb.zm], alpha[i], rho_l, rho_air);
                out = (float)((double)ws[f] - (double)bt * (pi - phi[nb.zm]) / hd);
            }
            wo[f] = out;
            const int ft = x + nx * (y + ny * nz);
            if (z == 0 && (g.periodic & 4)) wo[ft] = out;
            if (z == nz - 1 && !(g.periodic & 4)) {
                float top = 0.0f;
                if (outlet && ci != 0) top = (float)((double)ws[ft] + (double)gtop[x + nx * y] * pi / hd);
                wo[ft] = top;
            }
        }
        if (po) po[i] = ci != 0 ? (float)(p_scale * pi) : 0.0f;
    }
}

// max |div u| and sum div^2 over active cells of a face field.
__global__ void __launch_bounds__(TILE_THREADS) k_divergence(Grid3 g, float h, const uint8_t* __restrict__ cls,
                                                             const float* __restrict__ u, const float* __restrict__ v,
                                                             const float* __restrict__ w, Scalars* sc,
                                                             double* partials, int nblocks) {
    __shared__ double sh[8 * 2];
    double acc[2] = {0.0, 0.0};
    const int nx = g.nx, ny = g.ny;
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        if (cls[i] != 1) continue;
        double d = (double)u[x + 1 + (nx + 1) * (y + ny * z)] - (double)u[x + (nx + 1) * (y + ny * z)];
        d += (double)v[x + nx * (y + 1 + (ny + 1) * z)] - (double)v[x + nx * (y + (ny + 1) * z)];
        d += (double)w[x + nx * (y + ny * (z + 1))] - (double)w[x + nx * (y + ny * z)];
        d /= (double)h;
        acc[0] = fmax(acc[0], fabs(d));
        acc[1] += d * d;
    }
    // max via a separate warp/block path: reuse block_sum on -max trick is not
    // valid, so reduce the max explicitly.
    {
        const int t = threadIdx.x + blockDim.x * threadIdx.y;
        double m = warp_max(acc[0]);
        __shared__ double shm[8];
        if ((t & 31) == 0) shm[t >> 5] = m;
        __syncthreads();
        if (t < 32) {
            double mm = t < 8 ? shm[t] : 0.0;
            acc[0] = warp_max(mm);
        }
        __syncthreads();
    }
    {
        double s1[1] = {acc[1]};
        block_sum<1>(s1, sh);
        acc[1] = s1[0];
    }
    if (store_partials_is_last<2>(acc, partials, nblocks, &sc->ticket[5])) {
        __threadfence();
        const int t = threadIdx.x + blockDim.x * threadIdx.y;
        double m = 0.0, s = 0.0;
        for (int b = t; b < nblocks; b += TILE_THREADS) {
            m = fmax(m, ((volatile double*)partials)[b]);
            s += ((volatile double*)partials)[nblocks + b];
        }
        m = warp_max(m);
        __shared__ double shm2[8];
        if ((t & 31) == 0) shm2[t >> 5] = m;
        double s1[1] = {s};
        block_sum<1>(s1, sh);
        if (t == 0) {
            double mm = 0.0;
            for (int k = 0; k < 8; k++) mm = fmax(mm, shm2[k]);
            sc->divmax = mm;
            sc->div2 = s1[0];
            sc->ticket[5] = 0u;
        }
    }
}

// ----------------------------------------------------------- adjoint
// g_phi = d u / d phi ^T g_u + rho_l/dt g_p on active cells (the transposed
// gradient), FP64, into b64; ||b||^2.  Gradients of a periodic duplicate face
// are folded into the canonical face.
__global__ void __launch_bounds__(TILE_THREADS) k_adj_rhs(Grid3 g, int outlet, float h, float rho_l, float rho_air,
                                                          double p_scale, const uint8_t* __restrict__ cls,
                                                          const float* __restrict__ alpha,
                                                          const float* __restrict__ gtop,
                                                          const float* __restrict__ gu, const float* __restrict__ gv,
                                                          const float* __restrict__ gw, const float* __restrict__ gp,
                                                          double* __restrict__ b, Scalars* sc, double* partials,
                                                          int nblocks) {
    __shared__ double sh[8 * 1];
    double acc[1] = {0.0};
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const double inv_h = 1.0 / (double)h;
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        double s = 0.0;
        if (cls[i] == 1) {
            const Nbr nb = neighbours(g, x, y, z);
            const float ai = alpha[i];
            // x faces
            if (nb.xm >= 0 && cls[nb.xm] != 0) {
                double gf = gu[x + (nx + 1) * (y + ny * z)];
                if (x == 0) gf += gu[nx + (nx + 1) * (y + ny * z)];
                s -= (double)beta_of(alpha[nb.xm], ai, rho_l, rho_air) * inv_h * gf;
            }
            if (nb.xp >= 0 && cls[nb.xp] != 0) {
                const int hx = x + 1 == nx ? 0 : x + 1;
                double gf = gu[hx + (nx + 1) * (y + ny * z)];
                if (hx == 0) gf += gu[nx + (nx + 1) * (y + ny * z)];
                s += (double)beta_of(ai, alpha[nb.xp], rho_l, rho_air) * inv_h * gf;
            }
            if (nb.ym >= 0 && cls[nb.ym] != 0) {
                double gf = gv[x + nx * (y + (ny + 1) * z)];
                if (y == 0) gf += gv[x + nx * (ny + (ny + 1) * z)];
                s -= (double)beta_of(alpha[nb.ym], ai, rho_l, rho_air) * inv_h * gf;
            }
            if (nb.yp >= 0 && cls[nb.yp] != 0) {
                const int hy = y + 1 == ny ? 0 : y + 1;
                double gf = gv[x + nx * (hy + (ny + 1) * z)];
                if (hy == 0) gf += gv[x + nx * (ny + (ny + 1) * z)];
                s += (double)beta_of(ai, alpha[nb.yp], rho_l, rho_air) * inv_h * gf;
            }
            if (nb.zm >= 0 && cls[nb.zm] != 0) {
                double gf = gw[x + nx * (y + ny * z)];
                if (z == 0) gf += gw[x + nx * (y + ny * nz)];
                s -= (double)beta_of(alpha[nb.zm], ai, rho_l, rho_air) * inv_h * gf;
            }
            if (nb.zp >= 0 && cls[nb.zp] != 0) {
                const int hz = z + 1 == nz ? 0 : z + 1;
                double gf = gw[x + nx * (y + ny * hz)];
                if (hz == 0) gf += gw[x + nx * (y + ny * nz)];
                s += (double)beta_of(ai, alpha[nb.zp], rho_l, rho_air) * inv_h * gf;
            } else if (nb.zp < 0 && outlet && z == nz - 1) {
                s += (double)gtop[x + nx * y] * inv_h * (double)gw[x + nx * (y + ny * nz)];
            }
            if (gp) s += p_scale * (double)gp[i];
        }
        b[i] = s;
        acc[0] += s * s;
    }
    block_sum<1>(acc, sh);
    if (store_partials_is_last<1>(acc, partials, nblocks, &sc->ticket[0])) {
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
                                                              const double* __restrict__ psi,
                                                              const float* __restrict__ gu,
                                                              const float* __restrict__ gv,
                                                              const float* __restrict__ gw, float* __restrict__ ou,
                                                              float* __restrict__ ov, float* __restrict__ ow) {
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const double hd = (double)h;
    TILE_BEGIN(g) {
        if (!in_xy) continue;
        const int i = cell_index(g, x, y, z);
        const Nbr nb = neighbours(g, x, y, z);
        const uint8_t ci = cls[i];
        const double si = psi[i];
        {
            const int f = x + (nx + 1) * (y + ny * z), fd = nx + (nx + 1) * (y + ny * z);
            float out = 0.0f;
            if (nb.xm >= 0 && ci != 0 && cls[nb.xm] != 0) {
                double gf = gu[f];
                if (x == 0) gf += gu[fd];
                out = (float)(gf - hd * psi[nb.xm] + hd * si);
            }
            ou[f] = out;
            if (x == nx - 1) ou[fd] = 0.0f;
        }
        {
            const int f = x + nx * (y + (ny + 1) * z), fd = x + nx * (ny + (ny + 1) * z);
            float out = 0.0f;
            if (nb.ym >= 0 && ci != 0 && cls[nb.ym] != 0) {
                double gf = gv[f];
                if (y == 0) gf += gv[fd];
                out = (float)(gf - hd * psi[nb.ym] + hd * si);
            }
            ov[f] = out;
            if (y == ny - 1) ov[fd] = 0.0f;
        }
        {
            const int f = x + nx * (y + ny * z), fd = x + nx * (y + ny * nz);
            float out = 0.0f;
            if (nb.zm >= 0 && ci != 0 && cls[nb.zm] != 0) {
                double gf = gw[f];
                if (z == 0 && (g.periodic & 4)) gf += gw[fd];
                out = (float)(gf - hd * psi[nb.zm] + hd * si);
            }
            ow[f] = out;
            if (z == nz - 1) {
                float top = 0.0f;
                if (outlet && !(g.periodic & 4) && ci != 0) top = (float)((double)gw[fd] - hd * si);
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
// J = sum over outlet faces of w^2 (into sc->objective); seed_w = 2 w there.
__global__ void __launch_bounds__(TILE_THREADS) k_outlet_objective(Grid3 g, const float* __restrict__ w,
                                                                   float* __restrict__ seed_w, Scalars* sc,
                                                                   double* partials, int nblocks) {
    __shared__ double sh[8 * 1];
    double acc[1] = {0.0};
    const int x = blockIdx.x * TX + threadIdx.x;
    const int y = blockIdx.y * TY + threadIdx.y;
    if (x < g.nx && y < g.ny && blockIdx.z == 0) {
        const int ft = x + g.nx * (y + g.ny * g.nz);
        const double wz = w[ft];
        acc[0] = wz * wz;
        if (seed_w) seed_w[ft] = (float)(2.0 * wz);
    }
    block_sum<1>(acc, sh);
    if (store_partials_is_last<1>(acc, partials, nblocks, &sc->ticket[6])) {
        double tot[1];
        finish_partials<1>(tot, partials, nblocks, sh, &sc->ticket[6]);
        if (threadIdx.x == 0 && threadIdx.y == 0) sc->objective = tot[0];
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
    k_coefficients<<<L.grid, L.block, 0, s>>>(L.g, F.outlet, F.alpha, F.cls, F.rho_l, F.rho_air, F.coef, F.coef_lo,
                                              F.coef_lo_kind, F.gtop);
}
void launch_init_scalars(Scalars* sc, double tol2, double abs_floor, double inner_floor2, cudaStream_t s) {
    k_init_scalars<<<1, 1, 0, s>>>(sc, tol2, abs_floor, inner_floor2);
}
void launch_set_sigma(Scalars* sc, float sigma, cudaStream_t s) { k_set_sigma<<<1, 1, 0, s>>>(sc, sigma); }
void launch_rhs(const Launch& L, const Fields& F, const float* u, const float* v, const float* w, cudaStream_t s) {
    k_rhs<<<L.grid, L.block, 0, s>>>(L.g, F.outlet, F.h, F.cls, u, v, w, F.b64, F.sc, F.partials, L.nblocks);
}
void launch_residual64(const Launch& L, const Fields& F, const double* x64, cudaStream_t s) {
    k_residual64<<<L.grid, L.block, 0, s>>>(L.g, F.coef, F.b64, x64, F.r, F.e, F.sc, F.partials, L.nblocks,
                                            F.n_active);
}
void launch_spmv_pq(const Launch& L, const Fields& F, cudaStream_t s) {
    k_spmv_pq<<<L.grid, L.block, 0, s>>>(L.g, F.coef, F.p, F.q, F.sc, F.partials, L.nblocks);
}
void launch_update(const Launch& L, const Fields& F, cudaStream_t s) {
    k_update<<<L.grid, L.block, 0, s>>>(L.g, F.e, F.r, F.p, F.q, F.sc, F.partials, L.nblocks, F.n_active);
}
void launch_dot_rz(const Launch& L, const Fields& F, int init, cudaStream_t s) {
    k_dot_rz<<<L.grid, L.block, 0, s>>>(L.g, F.r, F.z, F.p, init, F.sc, F.partials, L.nblocks);
}
void launch_search(const Launch& L, const Fields& F, cudaStream_t s) {
    k_search<<<L.grid, L.block, 0, s>>>(L.g, F.z, F.p, F.sc);
}
void launch_accumulate(const Launch& L, const Fields& F, double* x64, cudaStream_t s) {
    k_accumulate<<<L.grid, L.block, 0, s>>>(L.g, x64, F.e);
}
void launch_correct(const Launch& L, const Fields& F, const double* phi, const float* us, const float* vs,
                    const float* ws, float* uo, float* vo, float* wo, float* po, float dt, cudaStream_t s) {
    const double p_scale = (double)F.rho_l / (double)dt;
    k_correct<<<L.grid, L.block, 0, s>>>(L.g, F.outlet, F.h, F.rho_l, F.rho_air, p_scale, F.cls, F.alpha, F.gtop, phi,
                                         us, vs, ws, uo, vo, wo, po);
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
    const double p_scale = (double)F.rho_l / (double)dt;
    k_adj_rhs<<<L.grid, L.block, 0, s>>>(L.g, F.outlet, F.h, F.rho_l, F.rho_air, p_scale, F.cls, F.alpha, F.gtop, gu,
                                         gv, gw, gp, F.b64, F.sc, F.partials, L.nblocks);
}
void launch_adj_correct(const Launch& L, const Fields& F, const double* psi, const float* gu, const float* gv,
                        const float* gw, float* ou, float* ov, float* ow, cudaStream_t s) {
    k_adj_correct<<<L.grid, L.block, 0, s>>>(L.g, F.outlet, F.h, F.cls, psi, gu, gv, gw, ou, ov, ow);
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
void launch_outlet_objective(const Launch& L, const Fields& F, const float* w, float* seed_w, cudaStream_t s) {
    dim3 grid(L.grid.x, L.grid.y, 1);
    k_outlet_objective<<<grid, L.block, 0, s>>>(L.g, w, seed_w, F.sc, F.partials, (int)(grid.x * grid.y));
}

}  // namespace mhdproj
