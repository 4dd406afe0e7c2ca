// fine_kernels.cu -- the finest-level stencil kernels with shared-memory
// plane staging.
//
// A block owns a 32 x 8 (x, y) tile and marches it along z.  A ring of four
// plane slots in shared memory holds, per plane: the vector tile with a
// one-cell halo (34 x 10), the coefficient records of the tile plus its +x
// column and +y row (33 x 9; the high faces), and the right-hand side of the
// tile.  Planes are fetched with cp.async four steps ahead of the plane being
// computed, so every warp keeps global loads in flight while it computes from
// shared memory; each value is read from HBM once per block (halo re-reads
// hit L2).  Outside a closed boundary the copies are zero-filled, which gives
// the zero coefficient of a wall face; periodic axes wrap the source index.
//
// Red-black half-steps update the cells of one colour in place: a cell of
// that colour is never a neighbour of another cell of the same colour (odd
// periodic extents use the out-of-place variant), so the staged snapshots are
// the values every update must read.
#include "kernels.h"

namespace mhdproj {

namespace {
constexpr int EW = TX + 2, EH = TY + 2;  // vector tile with halo
constexpr int CW = TX + 1, CH = TY + 1;  // coefficient tile (own + high neighbours)
constexpr int PF = 4;     // prefetch distance in planes
constexpr int NSLOT = 8;  // ring slots: planes z-1 .. z+PF

__device__ __forceinline__ void cp_async4(void* smem, const void* gmem, bool valid) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    const int n = valid ? 4 : 0;
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem, bool valid) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    const int n = valid ? 8 : 0;
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, bool valid) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    const int n = valid ? 16 : 0;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_wait_pf() { asm volatile("cp.async.wait_group %0;\n" ::"n"(PF - 1) : "memory"); }
__device__ __forceinline__ void cp_wait0() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

template <int CK> struct CoefStore { using T = uint2; };
template <> struct CoefStore<0> { using T = float4; };

template <int CK> __device__ __forceinline__ float4 unpack(const typename CoefStore<CK>::T& v);
template <> __device__ __forceinline__ float4 unpack<0>(const float4& v) { return v; }
template <> __device__ __forceinline__ float4 unpack<1>(const uint2& u) {
    const __half2 a = *reinterpret_cast<const __half2*>(&u.x), b = *reinterpret_cast<const __half2*>(&u.y);
    const float2 fa = __half22float2(a), fb = __half22float2(b);
    return make_float4(fa.x, fa.y, fb.x, fb.y);
}
template <> __device__ __forceinline__ float4 unpack<2>(const uint2& u) {
    const __nv_bfloat162 a = *reinterpret_cast<const __nv_bfloat162*>(&u.x);
    const __nv_bfloat162 b = *reinterpret_cast<const __nv_bfloat162*>(&u.y);
    const float2 fa = __bfloat1622float2(a), fb = __bfloat1622float2(b);
    return make_float4(fa.x, fa.y, fb.x, fb.y);
}

// Wrapped or absent coordinate along one axis.
__device__ __forceinline__ int axis_src(int c, int n, bool periodic, bool* ok) {
    if (c < 0) {
        *ok = periodic;
        return periodic ? c + n : 0;
    }
    if (c >= n) {
        *ok = periodic;
        return periodic ? c - n : n - 1;
    }
    *ok = true;
    return c;
}

template <int CK, bool WANT_E, bool WANT_R>
struct Ring {
    using CT = typename CoefStore<CK>::T;
    float e[NSLOT][EH][EW];
    CT c[NSLOT][CH][CW];
    float r[NSLOT][TY][TX];
};

// A thread's share of the plane copies, resolved once per block: the
// in-plane source offset and x-y validity of each element it copies.  A plane
// fetch is then a handful of cp.async with one plane offset added.
struct Fetcher {
    int eoff[2], coff[2], roff;   // in-plane source offsets
    short eslot[2], cslot[2];     // destination element index within a slot
    bool eok[2], cok[2], rok, ehas[2], chas[2];
    long long sxy;
    int nz;
    bool pz;

    __device__ __forceinline__ Fetcher(const Grid3& g, int x0, int y0) {
        const int t = threadIdx.x + TX * threadIdx.y;
        sxy = (long long)g.nx * g.ny;
        nz = g.nz;
        pz = (g.periodic & 4) != 0;
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const int k = t + j * TILE_THREADS;
            ehas[j] = k < EH * EW;
            eslot[j] = (short)k;
            eok[j] = false;
            eoff[j] = 0;
            if (ehas[j]) {
                const int ty = k / EW, tx = k - ty * EW;
                bool okx, oky;
                const int sx = axis_src(x0 - 1 + tx, g.nx, g.periodic & 1, &okx);
                const int sy = axis_src(y0 - 1 + ty, g.ny, g.periodic & 2, &oky);
                eok[j] = okx && oky;
                eoff[j] = eok[j] ? sx + g.nx * sy : 0;
            }
            chas[j] = k < CH * CW;
            cslot[j] = (short)k;
            cok[j] = false;
            coff[j] = 0;
            if (chas[j]) {
                const int ty = k / CW, tx = k - ty * CW;
                bool okx, oky;
                const int sx = axis_src(x0 + tx, g.nx, g.periodic & 1, &okx);
                const int sy = axis_src(y0 + ty, g.ny, g.periodic & 2, &oky);
                cok[j] = okx && oky;
                coff[j] = cok[j] ? sx + g.nx * sy : 0;
            }
        }
        const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
        rok = x < g.nx && y < g.ny;
        roff = rok ? x + g.nx * y : 0;
    }

    template <int CK, bool WANT_E, bool WANT_R>
    __device__ __forceinline__ void fetch(Ring<CK, WANT_E, WANT_R>& R, int zz, int slot, const float* ev,
                                          const typename CoefStore<CK>::T* coef, const float* rv) const {
        bool okz;
        const int sz = axis_src(zz, nz, pz, &okz);
        const long long plane = (long long)sz * sxy;
        if (WANT_E) {
            float* dst = &R.e[slot][0][0];
#pragma unroll
            for (int j = 0; j < 2; j++)
                if (ehas[j]) {
                    const bool ok = eok[j] && okz;
                    cp_async4(dst + eslot[j], ev + (ok ? plane + eoff[j] : 0), ok);
                }
        }
        auto* cdst = &R.c[slot][0][0];
#pragma unroll
        for (int j = 0; j < 2; j++)
            if (chas[j]) {
                const bool ok = cok[j] && okz;
                const auto* src = coef + (ok ? plane + coff[j] : 0);
                if (CK == 0) cp_async16(cdst + cslot[j], src, ok);
                else cp_async8(cdst + cslot[j], src, ok);
            }
        if (WANT_R) {
            const bool ok = rok && zz >= 0 && zz < nz;
            cp_async4(&R.r[slot][threadIdx.y][threadIdx.x], rv + (ok ? plane + roff : 0), ok);
        }
    }
};

__device__ __forceinline__ int slot_of(int zz, int z0) { return (zz - z0 + 1) & (NSLOT - 1); }
static_assert(NSLOT >= PF + 2 && (NSLOT & (NSLOT - 1)) == 0, "ring must hold planes z-1 .. z+PF");
}  // namespace

// --------------------------------------------------------------- SpMV
template <int CKD>  // coefficient storage of the operator: always FP32 here
__global__ void __launch_bounds__(TILE_THREADS) k_spmv_staged(Grid3 g, const float4* __restrict__ coef,
                                                              const float* __restrict__ p, float* __restrict__ q,
                                                              Scalars* sc, double* partials, int nblocks) {
    if (sc->converged) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto& R = *reinterpret_cast<Ring<0, true, false>*>(smem_raw);
    __shared__ double sh[8];
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    const int z0 = blockIdx.z * g.zper, z1 = min(g.nz, z0 + g.zper);
    const bool inside = x < g.nx && y < g.ny;
    const int tx = threadIdx.x, ty = threadIdx.y;
    Acc acc;
    const Fetcher F(g, x0, y0);
    F.fetch(R, z0 - 1, slot_of(z0 - 1, z0), p, coef, nullptr);
    F.fetch(R, z0, slot_of(z0, z0), p, coef, nullptr);
    cp_commit();
#pragma unroll
    for (int k = 1; k < PF; k++) {
        if (z0 + k <= z1) F.fetch(R, z0 + k, slot_of(z0 + k, z0), p, coef, nullptr);
        cp_commit();
    }
    for (int z = z0; z < z1; z++) {
        if (z + PF <= z1) F.fetch(R, z + PF, slot_of(z + PF, z0), p, coef, nullptr);
        cp_commit();
        cp_wait_pf();
        __syncthreads();
        if (inside) {
            const int s = slot_of(z, z0), sm = slot_of(z - 1, z0), sp = slot_of(z + 1, z0);
            const float4 cc = R.c[s][ty][tx];
            const float bxh = R.c[s][ty][tx + 1].x, byh = R.c[s][ty + 1][tx].y, bzh = R.c[sp][ty][tx].z;
            const float pc = R.e[s][ty + 1][tx + 1];
            float qv = cc.w * pc;
            qv = fmaf(cc.x, pc - R.e[s][ty + 1][tx], qv);
            qv = fmaf(bxh, pc - R.e[s][ty + 1][tx + 2], qv);
            qv = fmaf(cc.y, pc - R.e[s][ty][tx + 1], qv);
            qv = fmaf(byh, pc - R.e[s][ty + 2][tx + 1], qv);
            qv = fmaf(cc.z, pc - R.e[sm][ty + 1][tx + 1], qv);
            qv = fmaf(bzh, pc - R.e[sp][ty + 1][tx + 1], qv);
            q[x + g.nx * (y + g.ny * z)] = qv;
            acc.add_prod(pc, qv);
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

// ------------------------------------------------------- smoother half-step
// Fine level: rhs = sigma * r (FP32), correction z (FP32), coefficients in the
// level precision.  ZERO: first half-step from zero (no vector staging).
template <int CK, bool ZERO, bool OUT>
__global__ void __launch_bounds__(TILE_THREADS) k_smooth_staged(Grid3 g, const void* __restrict__ coef_v,
                                                                const float* __restrict__ r, float* e, float* out,
                                                                int color, const Scalars* sc) {
    if (sc->converged) return;
    using CT = typename CoefStore<CK>::T;
    const CT* coef = reinterpret_cast<const CT*>(coef_v);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto& R = *reinterpret_cast<Ring<CK, !ZERO, true>*>(smem_raw);
    const float sigma = sc->sigma;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    const int z0 = blockIdx.z * g.zper, z1 = min(g.nz, z0 + g.zper);
    const bool inside = x < g.nx && y < g.ny;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const Fetcher F(g, x0, y0);
    F.fetch(R, z0 - 1, slot_of(z0 - 1, z0), e, coef, r);
    F.fetch(R, z0, slot_of(z0, z0), e, coef, r);
    cp_commit();
#pragma unroll
    for (int k = 1; k < PF; k++) {
        if (z0 + k <= z1) F.fetch(R, z0 + k, slot_of(z0 + k, z0), e, coef, r);
        cp_commit();
    }
    for (int z = z0; z < z1; z++) {
        if (z + PF <= z1) F.fetch(R, z + PF, slot_of(z + PF, z0), e, coef, r);
        cp_commit();
        cp_wait_pf();
        __syncthreads();
        if (inside) {
            const int i = x + g.nx * (y + g.ny * z);
            if (((x + y + z) & 1) == color) {
                const int s = slot_of(z, z0), sm = slot_of(z - 1, z0), sp = slot_of(z + 1, z0);
                const float4 cc = unpack<CK>(R.c[s][ty][tx]);
                const float bxh = unpack<CK>(R.c[s][ty][tx + 1]).x;
                const float byh = unpack<CK>(R.c[s][ty + 1][tx]).y;
                const float bzh = unpack<CK>(R.c[sp][ty][tx]).z;
                const float d = ((cc.x + bxh) + (cc.y + byh)) + ((cc.z + bzh) + cc.w);
                float val = 0.f;
                if (d > 0.f) {
                    const float rhs = sigma * R.r[s][ty][tx];
                    if (ZERO) {
                        val = rhs / d;
                    } else {
                        float acc = rhs;
                        acc = fmaf(cc.x, R.e[s][ty + 1][tx], acc);
                        acc = fmaf(bxh, R.e[s][ty + 1][tx + 2], acc);
                        acc = fmaf(cc.y, R.e[s][ty][tx + 1], acc);
                        acc = fmaf(byh, R.e[s][ty + 2][tx + 1], acc);
                        acc = fmaf(cc.z, R.e[sm][ty + 1][tx + 1], acc);
                        acc = fmaf(bzh, R.e[sp][ty + 1][tx + 1], acc);
                        val = acc / d;
                    }
                }
                if (OUT) out[i] = val;
                else e[i] = val;
            } else if (ZERO) {
                e[i] = 0.f;
            }
        }
        __syncthreads();
    }
    cp_wait0();
}

// -------------------------------------------------- residual + restriction
// rc[Q] = 1/4 sum over the 2x2x2 children of (sigma r - A z); the z pair is
// summed over two steps, the x pair by a shuffle, the y pair through shared
// memory.  Requires an even z run per block.
template <int CK, class VTc>
__global__ void __launch_bounds__(TILE_THREADS) k_restrict_staged(Grid3 g, Grid3 gc, const void* __restrict__ coef_v,
                                                                  const float* __restrict__ r,
                                                                  const float* __restrict__ e, VTc* __restrict__ rc,
                                                                  const Scalars* sc) {
    if (sc->converged) return;
    using CT = typename CoefStore<CK>::T;
    const CT* coef = reinterpret_cast<const CT*>(coef_v);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto& R = *reinterpret_cast<Ring<CK, true, true>*>(smem_raw);
    __shared__ float ypart[TY][TX];
    const float sigma = sc->sigma;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    const int z0 = blockIdx.z * g.zper, z1 = min(g.nz, z0 + g.zper);
    const bool inside = x < g.nx && y < g.ny;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const Fetcher F(g, x0, y0);
    F.fetch(R, z0 - 1, slot_of(z0 - 1, z0), e, coef, r);
    F.fetch(R, z0, slot_of(z0, z0), e, coef, r);
    cp_commit();
#pragma unroll
    for (int k = 1; k < PF; k++) {
        if (z0 + k <= z1) F.fetch(R, z0 + k, slot_of(z0 + k, z0), e, coef, r);
        cp_commit();
    }
    float part = 0.f;
    for (int z = z0; z < z1; z++) {
        if (z + PF <= z1) F.fetch(R, z + PF, slot_of(z + PF, z0), e, coef, r);
        cp_commit();
        cp_wait_pf();
        __syncthreads();
        if (inside) {
            const int s = slot_of(z, z0), sm = slot_of(z - 1, z0), sp = slot_of(z + 1, z0);
            const float4 cc = unpack<CK>(R.c[s][ty][tx]);
            const float bxh = unpack<CK>(R.c[s][ty][tx + 1]).x;
            const float byh = unpack<CK>(R.c[s][ty + 1][tx]).y;
            const float bzh = unpack<CK>(R.c[sp][ty][tx]).z;
            const float d = ((cc.x + bxh) + (cc.y + byh)) + ((cc.z + bzh) + cc.w);
            float nsum = 0.f;
            nsum = fmaf(cc.x, R.e[s][ty + 1][tx], nsum);
            nsum = fmaf(bxh, R.e[s][ty + 1][tx + 2], nsum);
            nsum = fmaf(cc.y, R.e[s][ty][tx + 1], nsum);
            nsum = fmaf(byh, R.e[s][ty + 2][tx + 1], nsum);
            nsum = fmaf(cc.z, R.e[sm][ty + 1][tx + 1], nsum);
            nsum = fmaf(bzh, R.e[sp][ty + 1][tx + 1], nsum);
            part += sigma * R.r[s][ty][tx] - (d * R.e[s][ty + 1][tx + 1] - nsum);
        }
        const bool last_of_pair = ((z - z0) & 1) || z + 1 == z1;
        if (last_of_pair) {
            float v = part + __shfl_xor_sync(0xffffffffu, part, 1);
            ypart[ty][tx] = v;
            __syncthreads();
            if (inside && !(tx & 1) && !(ty & 1)) {
                const float tot = v + ypart[ty + 1][tx];
                rc[(x >> 1) + gc.nx * ((y >> 1) + gc.ny * (z >> 1))] = from_f<VTc>(0.25f * tot);
            }
            part = 0.f;
        }
        __syncthreads();
    }
    cp_wait0();
}

// ------------------------------------------------------------ launchers
template <int CK>
static size_t ring_bytes(bool want_e, bool want_r) {
    (void)want_e;
    (void)want_r;
    return sizeof(Ring<CK, true, true>);
}

void launch_spmv_staged(const Launch& L, const Fields& F, cudaStream_t s) {
    k_spmv_staged<0><<<L.grid, L.block, sizeof(Ring<0, true, false>), s>>>(L.g, F.coef, F.p, F.q, F.sc, F.partials,
                                                                           L.nblocks);
}

template <int CK>
static void smooth_staged_impl(const Launch& L, const void* coef, const float* r, float* e, float* tmp, int color,
                               bool zero, bool out_of_place, const Scalars* sc, cudaStream_t s) {
    const size_t sm = ring_bytes<CK>(true, true);
    if (zero) k_smooth_staged<CK, true, false><<<L.grid, L.block, sm, s>>>(L.g, coef, r, e, e, color, sc);
    else if (!out_of_place) k_smooth_staged<CK, false, false><<<L.grid, L.block, sm, s>>>(L.g, coef, r, e, e, color, sc);
    else k_smooth_staged<CK, false, true><<<L.grid, L.block, sm, s>>>(L.g, coef, r, e, tmp, color, sc);
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
    k_restrict_staged<CK, VTc><<<L.grid, L.block, ring_bytes<CK>(true, true), s>>>(L.g, gc, coef, r, e, (VTc*)rc, sc);
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
    set((const void*)k_spmv_staged<0>, sizeof(Ring<0, true, false>));
    set((const void*)k_smooth_staged<0, true, false>, sizeof(Ring<0, true, true>));
    set((const void*)k_smooth_staged<0, false, false>, sizeof(Ring<0, true, true>));
    set((const void*)k_smooth_staged<0, false, true>, sizeof(Ring<0, true, true>));
    set((const void*)k_smooth_staged<1, true, false>, sizeof(Ring<1, true, true>));
    set((const void*)k_smooth_staged<1, false, false>, sizeof(Ring<1, true, true>));
    set((const void*)k_smooth_staged<1, false, true>, sizeof(Ring<1, true, true>));
    set((const void*)k_smooth_staged<2, true, false>, sizeof(Ring<2, true, true>));
    set((const void*)k_smooth_staged<2, false, false>, sizeof(Ring<2, true, true>));
    set((const void*)k_smooth_staged<2, false, true>, sizeof(Ring<2, true, true>));
    set((const void*)k_restrict_staged<0, float>, sizeof(Ring<0, true, true>));
    set((const void*)k_restrict_staged<1, __half>, sizeof(Ring<1, true, true>));
    set((const void*)k_restrict_staged<2, __nv_bfloat16>, sizeof(Ring<2, true, true>));
    return e;
}

}  // namespace mhdproj
