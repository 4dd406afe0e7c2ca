// tma_fused.cu -- the fused multigrid smoothing passes with planes staged by
// the Tensor Memory Accelerator.
//
// k_pre_tma and k_post_tma do the work of k_presmooth_restrict and
// k_prolong_postsmooth (fused_kernels.cu) with the same per-cell arithmetic
// in the same order, so every vector they write is bit-identical; the
// difference is how planes reach shared memory and how work is spread over
// the threads:
//
//  * One thread with no other task issues, per plane, one
//    cp.async.bulk.tensor copy of each input: the smoother records (a 4-D box
//    over the split rows: half-row columns, even/odd half, y, z), the level
//    vectors (3-D boxes of RH rows from x0-4 for FP32 and from x0-8 for
//    2-byte values, so the first coordinate stays 16-byte aligned) and, for
//    the post-smoothing pass, the coarse correction (48 x CRH coarse cells
//    from x0/2-8).  The copies of a plane complete on one mbarrier; two
//    mbarriers alternate between planes.  Cells outside the grid arrive as
//    zeros (the copy's out-of-bounds fill), which is the closed wall the
//    cp.async zero fill stood for.  No thread computes a global address for a
//    halo load, which removes most of the integer work of the cp.async
//    kernels.
//  * 384 threads (224 with FP32 records) take at most one task in every
//    stage (360 red/prolongation quads, 324 black quads, 256 tile quads).
//    The 16 interior quads of a staged row go to one half-warp, so its
//    shared-memory accesses are contiguous; the halo quads of all rows follow.
//  * Records and corrections sit in five-slot rings (planes zA-3 .. zA+1), so
//    a step needs two barriers instead of three: warps that finish the tile
//    stage of plane zA-2 go on to the next plane's red stage while others
//    are still busy.

// Only grids without periodic axes take these kernels (a copy box cannot
// wrap around an axis); the cp.async kernels serve the others.  Every wait
// on an mbarrier is bounded: when it runs out the block stops issuing
// copies, marks the solve as stalled and converged (the host reports a
// timeout), and finishes its loop without waiting again.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <mutex>

#include "kernels.h"
#include "fused_common.cuh"

namespace mhdproj {

namespace {
using namespace staged;
using namespace fused;

template <int CK>
struct TGeo {
    static constexpr int FTY = CK == 0 ? 8 : 16;       // tile rows
    static constexpr int RH = FTY + 4;                 // staged rows y0-2 .. y0+FTY+1
    static constexpr int NRED = RH * NQ;               // red / prolongation quads
    static constexpr int NBR = FTY + 2;                // black rows y0-1 .. y0+FTY
    static constexpr int NBLK = NBR * NQ;              // black quads
    static constexpr int NOWN = QX * FTY;              // tile quads
    static constexpr int NT = (NRED + 32) / 32 * 32;   // threads: one red task each, and a spare issuing thread
    static constexpr int CRH = FTY / 2 + 2;            // coarse rows y0/2-1 .. y0/2+FTY/2
    static constexpr int CW = 48;                      // coarse columns x0/2-8 .. x0/2+39
    static constexpr int NS = 5;                       // ring slots of records and corrections: zA-3 .. zA+1
    static constexpr int NP = 6;                       // planes of a run of two with its halo (whole-run passes)
    static_assert(NBLK <= NT && NOWN <= NT && NRED < NT, "one task per thread");
};
// Staged rows of a level vector: x0-4 .. x0+67 for FP32 (the first
// coordinate x0-4 is 16-byte aligned), x0-8 .. x0+71 for 2-byte values.
template <class VT>
struct VGeo {
    static constexpr int XS = sizeof(VT) == 4 ? 4 : 8;  // row starts at x0 - XS
    static constexpr int VW = sizeof(VT) == 4 ? 72 : 80;
    static constexpr int VX = XS - XO;                 // column of x0-4 in a staged row
};
constexpr int TMA_MIN_BLOCKS = 2;
constexpr int WAIT_LIMIT = 1 << 22;

// ------------------------------------------------------------- PTX wrappers
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_barrier_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
// Orders this thread's (and, after a barrier, the block's) generic-proxy
// accesses of shared memory before the copies it issues next.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* b, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* b, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for the phase of the given parity; false when it ran out.
__device__ __forceinline__ bool mbar_wait(unsigned long long* b, unsigned parity) {
    for (int i = 0; i < WAIT_LIMIT; i++)
        if (mbar_try_wait(b, parity)) return true;
    return false;
}
__device__ __forceinline__ void tma_3d(void* dst, const CUtensorMap* tm, int x, int y, int z, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<unsigned long long>(tm)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tma_4d(void* dst, const CUtensorMap* tm, int x, int h, int y, int z,
                                       unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];\n" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<unsigned long long>(tm)), "r"(x), "r"(h), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

template <class T, int N>
constexpr int padded128() {  // elements of N T rounded up to 128 bytes
    return (int)(((N * sizeof(T) + 127) / 128) * 128 / sizeof(T));
}

// Shared memory of the pre-smoothing pass: records and corrections of planes
// zA-3 .. zA+1 (five slots), the copied residual and q of planes zA, zA+1.
template <int CK, class VT, bool UPDATE>
struct PreTmaSm {
    using CT = typename CoefStore<CK>::T;
    using G = TGeo<CK>;
    using V = VGeo<VT>;
    using VQ = VGeo<float>;
    alignas(128) CT c[G::NS][G::RH][RW];
    alignas(128) VT rv[2][G::RH][V::VW];
    alignas(128) float qv[UPDATE ? 2 : 1][UPDATE ? G::RH : 1][VQ::VW];
    alignas(16) float er[G::NS][G::RH][RW];
    float2 ypart[G::FTY][QX];
    unsigned long long bar[2];
    int abort_;
};
// Shared memory of the post-smoothing pass: records and smoothed corrections
// of planes zA-3 .. zA+1, the copied pre-smoothed correction and right-hand
// side of planes zA, zA+1, and the coarse correction of the two coarse
// planes they fall in.
template <int CK, class VT, class VTc>
struct PostTmaSm {
    using CT = typename CoefStore<CK>::T;
    using G = TGeo<CK>;
    using V = VGeo<VT>;
    static constexpr int ECS = padded128<VTc, G::CRH * G::CW>();
    alignas(128) CT c[G::NS][G::RH][RW];
    alignas(128) VT ev[2][G::RH][V::VW];
    alignas(128) VT rv[2][G::RH][V::VW];
    alignas(128) VTc ec[2][ECS];
    alignas(16) float ep[G::NS][G::RH][RW];
    unsigned long long bar[2];
    int abort_;
};
template <class SM>
__device__ __forceinline__ SM& aligned_smem(unsigned char* raw) {
    return *reinterpret_cast<SM*>(raw + ((128u - (smem_u32(raw) & 127u)) & 127u));
}

// Task of thread t in a stage over `rows` staged rows starting at row0: the
// 16 interior quads (1 .. 16) of a row go to one half-warp, so its
// shared-memory accesses are contiguous and free of bank conflicts; the two
// halo quads of each row (0 and 17) follow as tasks rows*16 .. rows*18-1.
__device__ __forceinline__ void stage_task(int t, int rows, int row0, int* row, int* q) {
    if (t < rows * 16) {
        *row = row0 + (t >> 4);
        *q = 1 + (t & 15);
    } else {
        const int e = t - rows * 16;
        *row = row0 + (e >> 1);
        *q = (e & 1) ? NQ - 1 : 0;
    }
}

// ------------------------------------------------------ pre-smoothing pass
// See k_presmooth_restrict for the algebra; rin and q arrive through tm_r
// and tm_q, the records through tm_rec.  A step handles the red stage of
// plane zA, the black stage of zA-1 and the tile stage of zA-2 with two
// barriers: the five-slot rings let the next step's copies and red stage
// start while other warps still finish the tile stage.
template <int CK, class VT, class VTc, bool UPDATE, bool FINE>
__global__ void __launch_bounds__(TGeo<CK>::NT, TMA_MIN_BLOCKS)
    k_pre_tma(const __grid_constant__ CUtensorMap tm_rec, const __grid_constant__ CUtensorMap tm_r,
              const __grid_constant__ CUtensorMap tm_q, Grid3 g, Grid3 gc, float* __restrict__ r_out,
              VT* __restrict__ e, VTc* __restrict__ rc, Scalars* sc, double* partials, int nblocks) {
    if (sc->converged) return;
    using CT = typename CoefStore<CK>::T;
    using G = TGeo<CK>;
    using V = VGeo<VT>;
    using VQ = VGeo<float>;
    using SM = PreTmaSm<CK, VT, UPDATE>;
    using R4 = typename Raw4<VT>::T;
    constexpr int FTY = G::FTY, NT = G::NT, RH = G::RH, NS = G::NS, SL = RH * RW;
    constexpr unsigned BYTES =
        RH * RW * sizeof(CT) + RH * V::VW * sizeof(VT) + (UPDATE ? RH * VQ::VW * 4 : 0);
    extern __shared__ __align__(128) unsigned char smem_raw[];
    SM& S = aligned_smem<SM>(smem_raw);
    __shared__ double sh[NT / 32];
    const int t = threadIdx.x;
    constexpr int ISSUER = NT - 1;  // no task in any stage
    const float sigma = FINE ? sc->sigma : 1.0f;
    const float alpha = UPDATE ? sc->alpha_f : 0.0f;
    const int x0 = blockIdx.x * PX, y0 = blockIdx.y * FTY;
    const int z0 = blockIdx.z * g.zper, z1 = min(g.nz, z0 + g.zper);
    const int zs = z0 - 2, nsteps = z1 - z0 + 4;  // planes zs .. z1+1
    const long long sxy = (long long)g.nx * g.ny;
    int last_issued = 0;
    auto issue = [&](int k, int off) {  // the copies of plane zs + k
        const int zz = zs + k;
        unsigned long long* b = &S.bar[k & 1];
        fence_proxy_async();
        mbar_expect_tx(b, BYTES);
        tma_4d(&S.c[0][0][0] + off, &tm_rec, 2 * x0 - 8, 0, y0 - 2, zz, b);
        tma_3d(&S.rv[k & 1][0][0], &tm_r, x0 - V::XS, y0 - 2, zz, b);
        if (UPDATE) tma_3d(&S.qv[k & 1][0][0], &tm_q, x0 - VQ::XS, y0 - 2, zz, b);
        last_issued = k;
    };
    if (t == ISSUER) {
        mbar_init(&S.bar[0], 1);
        mbar_init(&S.bar[1], 1);
        S.abort_ = 0;
        fence_barrier_init();
    }
    __syncthreads();
    if (t == ISSUER) issue(0, 0);

    // red task
    int r_row, r_q;
    stage_task(t, RH, 0, &r_row, &r_q);
    const bool has_red = t < G::NRED;
    const int r_o = r_row * RW + 2 * r_q;             // split offset of the quad's even half
    const int r_v = r_row * V::VW + V::VX + 4 * r_q;  // its cells in a copied vector row
    const int r_qv = r_row * VQ::VW + VQ::VX + 4 * r_q;
    const int r_gx = x0 - XO + 4 * r_q, r_gy = y0 - 2 + r_row;
    const int r_par = r_gy & 1;
    const int r_own = (has_red && r_row >= 2 && r_row < FTY + 2 && r_q >= 1 && r_q <= QX && r_gx < g.nx && r_gy < g.ny)
                          ? r_gx + g.nx * r_gy
                          : -1;
    // black task
    int b_row, b_q;
    stage_task(t, G::NBR, 1, &b_row, &b_q);
    const bool has_blk = t < G::NBLK;
    const int b_o = b_row * RW + 2 * b_q;
    const int b_par = (y0 - 2 + b_row) & 1;
    // tile task: the own quad
    const bool has_own = t < G::NOWN;
    const int tx = t % QX, ty = t / QX;
    const int ox = x0 + 4 * tx, oy = y0 + ty;
    const bool own_inside = has_own && ox < g.nx && oy < g.ny;
    const int oo = (ty + 2) * RW + 2 * (tx + 1);
    const long long og = ox + (long long)g.nx * oy;

    const CT* c0 = &S.c[0][0][0];
    float* e0 = &S.er[0][0][0];
    float rr_thread = 0.f;
    float2 part = make_float2(0.f, 0.f);
    int rc_z = -1;
    auto flush_rc = [&]() {
        if (rc_z >= 0 && own_inside && !(ty & 1)) {
            const float2 a = S.ypart[ty][tx], b = S.ypart[ty + 1][tx];
            st2<VTc>(rc + (ox >> 1) + (long long)gc.nx * ((oy >> 1) + (long long)gc.ny * rc_z),
                     make_float2(0.25f * (a.x + b.x), 0.25f * (a.y + b.y)));
        }
        rc_z = -1;
    };
    // element offsets of the ring slots of planes zA, zA-1, zA-2, zA-3
    int o0 = 0, o1 = (NS - 1) * SL, o2 = (NS - 2) * SL, o3 = (NS - 3) * SL;
    auto step = [&](auto ph, int k) {
        constexpr int P = decltype(ph)::value;  // k & 3; zs is even, so plane zA has parity P & 1
        const int zA = zs + k;
        const bool aborted = *reinterpret_cast<volatile int*>(&S.abort_) != 0;
        if (t == ISSUER && k + 1 < nsteps && !aborted) issue(k + 1, o0 == (NS - 1) * SL ? 0 : o0 + SL);
        if (!aborted && !mbar_wait(&S.bar[P & 1], P >> 1)) {
            S.abort_ = 1;
            sc->stalled = 1;
            sc->converged = 1;
        }
        // ---- red stage: plane zA over the 2-halo rows
        if (has_red) {
            const CT* C = c0 + o0;
            float* ER = e0 + o0;
            float4 rn = cvt4r<VT>(*reinterpret_cast<const R4*>(&S.rv[P & 1][0][0] + r_v));
            if (UPDATE) {
                const float4 qq = *reinterpret_cast<const float4*>(&S.qv[P & 1][0][0] + r_qv);
                rn = make_float4(fmaf(-alpha, qq.x, rn.x), fmaf(-alpha, qq.y, rn.y), fmaf(-alpha, qq.z, rn.z),
                                 fmaf(-alpha, qq.w, rn.w));
            }
            const int p = r_par ^ (P & 1);
            float4 d0, d1;
            rec2<CK>(C + r_o + p * HW, &d0, &d1);
            const float2 rr = p ? make_float2(rn.y, rn.w) : make_float2(rn.x, rn.z);  // red cells
            const float2 rb = p ? make_float2(rn.x, rn.z) : make_float2(rn.y, rn.w);  // black cells
            const float2 ev = divide2(make_float2(sigma * rr.x, sigma * rr.y), make_float2(d0.w, d1.w));
            *reinterpret_cast<float2*>(ER + r_o + p * HW) = ev;
            *reinterpret_cast<float2*>(ER + r_o + (1 - p) * HW) = make_float2(sigma * rb.x, sigma * rb.y);
            if (UPDATE && r_own >= 0 && zA >= z0 && zA < z1) {
                *reinterpret_cast<float4*>(r_out + sxy * zA + r_own) = rn;
                rr_thread = fmaf(rn.x, rn.x, fmaf(rn.y, rn.y, fmaf(rn.z, rn.z, fmaf(rn.w, rn.w, rr_thread))));
            }
        }
        __syncthreads();
        flush_rc();
        // ---- black stage: plane zA-1 over the 1-halo rows, in place
        if (has_blk && zA - 1 >= z0 - 1) {
            const CT* C = c0 + o1;
            const CT* CN = c0 + o0;
            float* E = e0 + o1;
            const float* EM = e0 + o2;
            const float* EP = e0 + o0;
            const int h = b_par ^ (P & 1);  // black half of the row at plane zA-1
            const int o = b_o + h * HW;
            float2 d;
            const float2 s = gs_sum2<CK>(C, CN, E, EM, EP, o, h, *reinterpret_cast<const float2*>(E + o), &d);
            *reinterpret_cast<float2*>(E + o) = divide2(s, d);
        }
        __syncthreads();
        // ---- correction out and restriction: plane zA-2 over the tile
        const int zC = zA - 2;
        if (has_own && zC >= z0 && zC < z1) {
            const CT* C = c0 + o2;
            const CT* CN = c0 + o1;
            const float* E = e0 + o2;
            const float* EM = e0 + o3;
            const float* EP = e0 + o1;
            const int p = (oy & 1) ^ (P & 1);  // red half of the own quad
            float2 d;
            const float2 s = gs_sum2<CK>(C, CN, E, EM, EP, oo + p * HW, p, make_float2(0.f, 0.f), &d);
            part.x += s.x;
            part.y += s.y;
            if (own_inside) {
                const float2 ev = *reinterpret_cast<const float2*>(E + oo);
                const float2 od = *reinterpret_cast<const float2*>(E + oo + HW);
                st4<VT>(e + (og + sxy * zC), make_float4(ev.x, od.x, ev.y, od.y));
            }
            if ((zC & 1) || zC + 1 == z1) {
                // the row pair sum is formed after the next step's first barrier
                S.ypart[ty][tx] = part;
                rc_z = zC >> 1;
                part = make_float2(0.f, 0.f);
            }
        }
    };
    auto advance = [&]() {
        o3 = o2;
        o2 = o1;
        o1 = o0;
        o0 = o0 == (NS - 1) * SL ? 0 : o0 + SL;
    };
    for (int k = 0;;) {
        step(Phase<0>{}, k);
        advance();
        if (++k >= nsteps) break;
        step(Phase<1>{}, k);
        advance();
        if (++k >= nsteps) break;
        step(Phase<2>{}, k);
        advance();
        if (++k >= nsteps) break;
        step(Phase<3>{}, k);
        advance();
        if (++k >= nsteps) break;
    }
    __syncthreads();
    flush_rc();
    if (t == ISSUER && S.abort_) (void)mbar_wait(&S.bar[last_issued & 1], (last_issued >> 1) & 1);
    if (UPDATE) {
        double v1[1] = {(double)rr_thread};
        block_sum<1>(v1, sh);
        if (store_partials_is_last<1>(v1, partials, nblocks, &sc->ticket[8])) {
            double tot[1];
            finish_partials<1>(tot, partials, nblocks, sh, &sc->ticket[8]);
            if (t == 0 && !sc->stalled) {
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
// See k_prolong_postsmooth; e, r and the coarse correction arrive through
// tm_e, tm_r and tm_ec, the records through tm_rec.  Step structure as in
// k_pre_tma.
template <int CK, class VT, class VTc, bool DOT, bool FINE>
__global__ void __launch_bounds__(TGeo<CK>::NT, TMA_MIN_BLOCKS)
    k_post_tma(const __grid_constant__ CUtensorMap tm_rec, const __grid_constant__ CUtensorMap tm_e,
               const __grid_constant__ CUtensorMap tm_r, const __grid_constant__ CUtensorMap tm_ec, Grid3 g,
               VT* __restrict__ out, const VT* __restrict__ accum, float w, Scalars* sc, double* partials,
               int nblocks, long long n_active) {
    if (sc->converged) return;
    using CT = typename CoefStore<CK>::T;
    using G = TGeo<CK>;
    using V = VGeo<VT>;
    using SM = PostTmaSm<CK, VT, VTc>;
    using R4 = typename Raw4<VT>::T;
    using C2 = typename Raw2<VTc>::T;
    constexpr int FTY = G::FTY, NT = G::NT, RH = G::RH, NS = G::NS, SL = RH * RW;
    constexpr unsigned BYTES = RH * RW * sizeof(CT) + 2 * RH * V::VW * sizeof(VT);
    constexpr unsigned EC_BYTES = G::CRH * G::CW * sizeof(VTc);
    extern __shared__ __align__(128) unsigned char smem_raw[];
    SM& S = aligned_smem<SM>(smem_raw);
    __shared__ double sh[NT / 32];
    const int t = threadIdx.x;
    constexpr int ISSUER = NT - 1;
    const float sigma = FINE ? sc->sigma : 1.0f;
    const float is = FINE ? sc->inv_sigma : 1.0f;
    const int x0 = blockIdx.x * PX, y0 = blockIdx.y * FTY;
    const int z0 = blockIdx.z * g.zper, z1 = min(g.nz, z0 + g.zper);
    const int zs = z0 - 2, nsteps = z1 - z0 + 4;
    const long long sxy = (long long)g.nx * g.ny;
    int last_issued = 0;
    auto issue = [&](int k, int off) {  // the copies of plane zs + k (and its coarse plane when it starts one)
        const int zz = zs + k;
        unsigned long long* b = &S.bar[k & 1];
        fence_proxy_async();
        mbar_expect_tx(b, BYTES + ((k & 1) ? 0u : EC_BYTES));
        tma_4d(&S.c[0][0][0] + off, &tm_rec, 2 * x0 - 8, 0, y0 - 2, zz, b);
        tma_3d(&S.ev[k & 1][0][0], &tm_e, x0 - V::XS, y0 - 2, zz, b);
        tma_3d(&S.rv[k & 1][0][0], &tm_r, x0 - V::XS, y0 - 2, zz, b);
        if (!(k & 1)) tma_3d(&S.ec[(k >> 1) & 1][0], &tm_ec, (x0 >> 1) - 8, (y0 >> 1) - 1, zz >> 1, b);
        last_issued = k;
    };
    if (t == ISSUER) {
        mbar_init(&S.bar[0], 1);
        mbar_init(&S.bar[1], 1);
        S.abort_ = 0;
        fence_barrier_init();
    }
    __syncthreads();
    if (t == ISSUER) issue(0, 0);

    int r_row, r_q;
    stage_task(t, RH, 0, &r_row, &r_q);
    const bool has_red = t < G::NRED;
    const int r_o = r_row * RW + 2 * r_q;
    const int r_v = r_row * V::VW + V::VX + 4 * r_q;
    const int r_c = (r_row >> 1) * G::CW + 6 + 2 * r_q;  // the quad's two coarse parents
    const int r_gx = x0 - XO + 4 * r_q, r_gy = y0 - 2 + r_row;
    const int r_par = r_gy & 1;
    const bool r_inside = r_gx >= 0 && r_gx < g.nx && r_gy >= 0 && r_gy < g.ny;
    int b_row, b_q;
    stage_task(t, G::NBR, 1, &b_row, &b_q);
    const bool has_blk = t < G::NBLK;
    const int b_o = b_row * RW + 2 * b_q;
    const int b_par = (y0 - 2 + b_row) & 1;
    const bool has_own = t < G::NOWN;
    const int tx = t % QX, ty = t / QX;
    const int ox = x0 + 4 * tx, oy = y0 + ty;
    const bool own_inside = has_own && ox < g.nx && oy < g.ny;
    const int oo = (ty + 2) * RW + 2 * (tx + 1);
    const int ov = (ty + 2) * V::VW + V::VX + 4 * (tx + 1);
    const long long og = ox + (long long)g.nx * oy;
    const CT* c0 = &S.c[0][0][0];
    float* e0 = &S.ep[0][0][0];
    Acc acc;
    R4 rq_own[4];  // own quad's right-hand side of planes zA-3 .. zA (slot zA & 3)

    int o0 = 0, o1 = (NS - 1) * SL, o2 = (NS - 2) * SL, o3 = (NS - 3) * SL;
    auto step = [&](auto ph, int k) {
        constexpr int P = decltype(ph)::value;
        const int zA = zs + k;
        const bool aborted = *reinterpret_cast<volatile int*>(&S.abort_) != 0;
        if (t == ISSUER && k + 1 < nsteps && !aborted) issue(k + 1, o0 == (NS - 1) * SL ? 0 : o0 + SL);
        if (!aborted && !mbar_wait(&S.bar[P & 1], P >> 1)) {
            S.abort_ = 1;
            sc->stalled = 1;
            sc->converged = 1;
        }
        if (has_own) rq_own[P] = *reinterpret_cast<const R4*>(&S.rv[P & 1][0][0] + ov);
        // ---- prolongation: plane zA over the 2-halo rows
        if (has_red) {
            float* EP = e0 + o0;
            float4 ev = make_float4(0.f, 0.f, 0.f, 0.f), rq = ev;
            float2 cv = make_float2(0.f, 0.f);
            if (r_inside && zA >= 0 && zA < g.nz) {
                ev = cvt4r<VT>(*reinterpret_cast<const R4*>(&S.ev[P & 1][0][0] + r_v));
                rq = cvt4r<VT>(*reinterpret_cast<const R4*>(&S.rv[P & 1][0][0] + r_v));
                cv = cvt2(*reinterpret_cast<const C2*>(&S.ec[P >> 1][0] + r_c));
            }
            const int p = r_par ^ (P & 1);
            const float2 er = p ? make_float2(ev.y, ev.w) : make_float2(ev.x, ev.z);
            const float2 rb = p ? make_float2(rq.x, rq.z) : make_float2(rq.y, rq.w);
            *reinterpret_cast<float2*>(EP + r_o + p * HW) = make_float2(fmaf(w, cv.x, er.x), fmaf(w, cv.y, er.y));
            *reinterpret_cast<float2*>(EP + r_o + (1 - p) * HW) = make_float2(sigma * rb.x, sigma * rb.y);
        }
        __syncthreads();
        // ---- black half-step: plane zA-1 over the 1-halo rows, in place
        if (has_blk && zA - 1 >= z0 - 1) {
            const CT* C = c0 + o1;
            const CT* CN = c0 + o0;
            float* E = e0 + o1;
            const float* EM = e0 + o2;
            const float* EP = e0 + o0;
            const int h = b_par ^ (P & 1);
            const int o = b_o + h * HW;
            float2 d;
            const float2 s = gs_sum2<CK>(C, CN, E, EM, EP, o, h, *reinterpret_cast<const float2*>(E + o), &d);
            *reinterpret_cast<float2*>(E + o) = divide2(s, d);
        }
        __syncthreads();
        // ---- red half-step: plane zA-2 over the tile, out = z
        const int zC = zA - 2;
        if (has_own && zC >= z0 && zC < z1) {
            const CT* C = c0 + o2;
            const CT* CN = c0 + o1;
            const float* E = e0 + o2;
            const float* EM = e0 + o3;
            const float* EP = e0 + o1;
            const int p = (oy & 1) ^ (P & 1);
            const float4 rv = cvt4r<VT>(rq_own[(P + 2) & 3]);
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
    auto advance = [&]() {
        o3 = o2;
        o2 = o1;
        o1 = o0;
        o0 = o0 == (NS - 1) * SL ? 0 : o0 + SL;
    };
    for (int k = 0;;) {
        step(Phase<0>{}, k);
        advance();
        if (++k >= nsteps) break;
        step(Phase<1>{}, k);
        advance();
        if (++k >= nsteps) break;
        step(Phase<2>{}, k);
        advance();
        if (++k >= nsteps) break;
        step(Phase<3>{}, k);
        advance();
        if (++k >= nsteps) break;
    }
    __syncthreads();
    if (t == ISSUER && S.abort_) (void)mbar_wait(&S.bar[last_issued & 1], (last_issued >> 1) & 1);
    if (DOT) {
        double v1[1] = {acc.total()};
        block_sum<1>(v1, sh);
        if (store_partials_is_last<1>(v1, partials, nblocks, &sc->ticket[9])) {
            double tot[1];
            finish_partials<1>(tot, partials, nblocks, sh, &sc->ticket[9]);
            if (t == 0 && !sc->stalled) {
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
                sc->inv_sigma_z = sc->inv_sigma;
                set_sigma_from(sc, sc->rr, n_active);
            }
        }
    }
}

// ------------------------------------------------- whole-run coarse passes
// On a coarse level whose runs of two planes fill at most one wave of one
// block per SM (the 64^3 and 32^3 levels below a 256^3 or 128^3 grid), a
// z-marching pass is six plane steps of three dependent stages each, and the
// stages' latency, not bandwidth, sets its time.  These kernels do the same
// work with each stage over every plane of the run at once: the red (or
// prolongation) stage over planes z0-2 .. z1+1, the black half-step over
// z0-1 .. z1, the restriction (or last red half-step) over z0 .. z1-1, with a
// barrier between stages.  Every plane's copies are issued when the block
// starts, each plane on its own mbarrier.  The per-cell arithmetic and its
// order are those of k_pre_tma / k_post_tma on coarse levels, so every
// vector written is bit-identical.
template <int CK, class VT>
struct PreRunSm {
    using CT = typename CoefStore<CK>::T;
    using G = TGeo<CK>;
    using V = VGeo<VT>;
    alignas(128) CT c[G::NP][G::RH][RW];
    alignas(128) VT rv[G::NP][G::RH][V::VW];
    alignas(16) float er[G::NP][G::RH][RW];
    float2 ypart[G::FTY][QX];
    unsigned long long bar[G::NP];
    int abort_;
};
template <int CK, class VT, class VTc>
struct PostRunSm {
    using CT = typename CoefStore<CK>::T;
    using G = TGeo<CK>;
    using V = VGeo<VT>;
    static constexpr int ECS = padded128<VTc, G::CRH * G::CW>();
    alignas(128) CT c[G::NP][G::RH][RW];
    alignas(128) VT ev[G::NP][G::RH][V::VW];
    alignas(128) VT rv[G::NP][G::RH][V::VW];
    alignas(128) VTc ec[G::NP / 2][ECS];
    alignas(16) float ep[G::NP][G::RH][RW];
    unsigned long long bar[G::NP];
    int abort_;
};

// Issue the copies of planes zs .. zs+np-1 (thread ISSUER) and wait for all of
// them (every thread, bounded); false when a wait ran out.
template <class SM, class IssueFn>
__device__ __forceinline__ bool run_copies(SM& S, int np, int issuer, IssueFn issue_plane) {
    const int t = threadIdx.x;
    if (t == issuer) {
        for (int k = 0; k < (int)(sizeof(S.bar) / sizeof(S.bar[0])); k++) mbar_init(&S.bar[k], 1);
        S.abort_ = 0;
        fence_barrier_init();
    }
    __syncthreads();
    if (t == issuer)
        for (int k = 0; k < np; k++) issue_plane(k, &S.bar[k]);
    bool ok = true;
    for (int k = 0; k < np && ok; k++) ok = mbar_wait(&S.bar[k], 0);
    return ok;
}
// After a timed-out wait: the issuing thread waits (bounded) for every copy
// it issued before the block exits.
template <class SM>
__device__ __forceinline__ void run_drain(SM& S, int np, int issuer) {
    if (threadIdx.x == issuer && S.abort_)
        for (int k = 0; k < np; k++) (void)mbar_wait(&S.bar[k], 0);
}

template <int CK, class VT, class VTc>
__global__ void __launch_bounds__(TGeo<CK>::NT, 1)
    k_pre_run(const __grid_constant__ CUtensorMap tm_rec, const __grid_constant__ CUtensorMap tm_r, Grid3 g,
              Grid3 gc, VT* __restrict__ e, VTc* __restrict__ rc, Scalars* sc) {
    if (sc->converged) return;
    using CT = typename CoefStore<CK>::T;
    using G = TGeo<CK>;
    using V = VGeo<VT>;
    using SM = PreRunSm<CK, VT>;
    using R4 = typename Raw4<VT>::T;
    constexpr int FTY = G::FTY, NT = G::NT, RH = G::RH, NP = G::NP, SL = RH * RW;
    constexpr unsigned BYTES = RH * RW * sizeof(CT) + RH * V::VW * sizeof(VT);
    extern __shared__ __align__(128) unsigned char smem_raw[];
    SM& S = aligned_smem<SM>(smem_raw);
    const int t = threadIdx.x;
    constexpr int ISSUER = NT - 1;
    const int x0 = blockIdx.x * PX, y0 = blockIdx.y * FTY;
    const int z0 = blockIdx.z * 2, z1 = min(g.nz, z0 + 2);
    const int zs = z0 - 2, np = z1 - z0 + 4;  // planes zs .. z1+1; zs is even
    const long long sxy = (long long)g.nx * g.ny;
    const bool ok = run_copies(S, np, ISSUER, [&](int k, unsigned long long* b) {
        fence_proxy_async();
        mbar_expect_tx(b, BYTES);
        tma_4d(&S.c[k][0][0], &tm_rec, 2 * x0 - 8, 0, y0 - 2, zs + k, b);
        tma_3d(&S.rv[k][0][0], &tm_r, x0 - V::XS, y0 - 2, zs + k, b);
    });
    if (!ok) {
        S.abort_ = 1;
        sc->stalled = 1;
        sc->converged = 1;
    }
    const CT* c0 = &S.c[0][0][0];
    float* e0 = &S.er[0][0][0];
    // ---- red stage, planes 0 .. np-1 over the 2-halo rows
    if (ok && t < G::NRED) {
        int row, q;
        stage_task(t, RH, 0, &row, &q);
        const int o = row * RW + 2 * q, vo = row * V::VW + V::VX + 4 * q;
        const int par = (y0 - 2 + row) & 1;
#pragma unroll
        for (int k = 0; k < NP; k++) {
            if (k >= np) break;
            const float4 rn = cvt4r<VT>(*reinterpret_cast<const R4*>(&S.rv[k][0][0] + vo));
            const int p = par ^ (k & 1);
            float4 d0, d1;
            rec2<CK>(c0 + k * SL + o + p * HW, &d0, &d1);
            const float2 rr = p ? make_float2(rn.y, rn.w) : make_float2(rn.x, rn.z);
            const float2 rb = p ? make_float2(rn.x, rn.z) : make_float2(rn.y, rn.w);
            const float2 ev = divide2(make_float2(1.0f * rr.x, 1.0f * rr.y), make_float2(d0.w, d1.w));
            *reinterpret_cast<float2*>(e0 + k * SL + o + p * HW) = ev;
            *reinterpret_cast<float2*>(e0 + k * SL + o + (1 - p) * HW) = make_float2(1.0f * rb.x, 1.0f * rb.y);
        }
    }
    __syncthreads();
    // ---- black half-step, planes 1 .. np-2 over the 1-halo rows, in place
    if (ok && t < G::NBLK) {
        int row, q;
        stage_task(t, G::NBR, 1, &row, &q);
        const int ob = row * RW + 2 * q;
        const int par = (y0 - 2 + row) & 1;
#pragma unroll
        for (int k = 1; k < NP - 1; k++) {
            if (k > np - 2) break;
            const int h = par ^ ((k + 1) & 1);
            const int o = ob + h * HW;
            float* E = e0 + k * SL;
            float2 d;
            const float2 s = gs_sum2<CK>(c0 + k * SL, c0 + (k + 1) * SL, E, E - SL, E + SL, o, h,
                                         *reinterpret_cast<const float2*>(E + o), &d);
            *reinterpret_cast<float2*>(E + o) = divide2(s, d);
        }
    }
    __syncthreads();
    // ---- correction out and restriction, planes 2 .. np-3 over the tile
    const bool has_own = t < G::NOWN;
    const int tx = t % QX, ty = t / QX;
    const int ox = x0 + 4 * tx, oy = y0 + ty;
    const bool own_inside = has_own && ox < g.nx && oy < g.ny;
    const int oo = (ty + 2) * RW + 2 * (tx + 1);
    const long long og = ox + (long long)g.nx * oy;
    if (ok && has_own) {
        float2 part = make_float2(0.f, 0.f);
        for (int k = 2; k < np - 2; k++) {
            const int zC = zs + k;
            const float* E = e0 + k * SL;
            const int p = (oy & 1) ^ (k & 1);
            float2 d;
            const float2 s = gs_sum2<CK>(c0 + k * SL, c0 + (k + 1) * SL, E, E - SL, E + SL, oo + p * HW, p,
                                         make_float2(0.f, 0.f), &d);
            part.x += s.x;
            part.y += s.y;
            if (own_inside) {
                const float2 ev = *reinterpret_cast<const float2*>(E + oo);
                const float2 od = *reinterpret_cast<const float2*>(E + oo + HW);
                st4<VT>(e + (og + sxy * zC), make_float4(ev.x, od.x, ev.y, od.y));
            }
        }
        S.ypart[ty][tx] = part;
    }
    __syncthreads();
    if (ok && own_inside && !(ty & 1)) {
        const float2 a = S.ypart[ty][tx], b = S.ypart[ty + 1][tx];
        st2<VTc>(rc + (ox >> 1) + (long long)gc.nx * ((oy >> 1) + (long long)gc.ny * (z0 >> 1)),
                 make_float2(0.25f * (a.x + b.x), 0.25f * (a.y + b.y)));
    }
    run_drain(S, np, ISSUER);
}

template <int CK, class VT, class VTc>
__global__ void __launch_bounds__(TGeo<CK>::NT, 1)
    k_post_run(const __grid_constant__ CUtensorMap tm_rec, const __grid_constant__ CUtensorMap tm_e,
               const __grid_constant__ CUtensorMap tm_r, const __grid_constant__ CUtensorMap tm_ec, Grid3 g,
               VT* __restrict__ out, const VT* __restrict__ accum, float w, Scalars* sc) {
    if (sc->converged) return;
    using CT = typename CoefStore<CK>::T;
    using G = TGeo<CK>;
    using V = VGeo<VT>;
    using SM = PostRunSm<CK, VT, VTc>;
    using R4 = typename Raw4<VT>::T;
    using C2 = typename Raw2<VTc>::T;
    constexpr int FTY = G::FTY, NT = G::NT, RH = G::RH, NP = G::NP, SL = RH * RW;
    constexpr unsigned BYTES = RH * RW * sizeof(CT) + 2 * RH * V::VW * sizeof(VT);
    constexpr unsigned EC_BYTES = G::CRH * G::CW * sizeof(VTc);
    extern __shared__ __align__(128) unsigned char smem_raw[];
    SM& S = aligned_smem<SM>(smem_raw);
    const int t = threadIdx.x;
    constexpr int ISSUER = NT - 1;
    const int x0 = blockIdx.x * PX, y0 = blockIdx.y * FTY;
    const int z0 = blockIdx.z * 2, z1 = min(g.nz, z0 + 2);
    const int zs = z0 - 2, np = z1 - z0 + 4;
    const long long sxy = (long long)g.nx * g.ny;
    const bool ok = run_copies(S, np, ISSUER, [&](int k, unsigned long long* b) {
        const int zz = zs + k;
        fence_proxy_async();
        mbar_expect_tx(b, BYTES + ((k & 1) ? 0u : EC_BYTES));
        tma_4d(&S.c[k][0][0], &tm_rec, 2 * x0 - 8, 0, y0 - 2, zz, b);
        tma_3d(&S.ev[k][0][0], &tm_e, x0 - V::XS, y0 - 2, zz, b);
        tma_3d(&S.rv[k][0][0], &tm_r, x0 - V::XS, y0 - 2, zz, b);
        if (!(k & 1)) tma_3d(&S.ec[k >> 1][0], &tm_ec, (x0 >> 1) - 8, (y0 >> 1) - 1, zz >> 1, b);
    });
    if (!ok) {
        S.abort_ = 1;
        sc->stalled = 1;
        sc->converged = 1;
    }
    const CT* c0 = &S.c[0][0][0];
    float* e0 = &S.ep[0][0][0];
    // ---- prolongation, planes 0 .. np-1 over the 2-halo rows
    if (ok && t < G::NRED) {
        int row, q;
        stage_task(t, RH, 0, &row, &q);
        const int o = row * RW + 2 * q, vo = row * V::VW + V::VX + 4 * q;
        const int co = (row >> 1) * G::CW + 6 + 2 * q;  // the quad's two coarse parents
        const int gx = x0 - XO + 4 * q, gy = y0 - 2 + row;
        const int par = gy & 1;
        const bool inside = gx >= 0 && gx < g.nx && gy >= 0 && gy < g.ny;
#pragma unroll
        for (int k = 0; k < NP; k++) {
            if (k >= np) break;
            const int zA = zs + k;
            float4 ev = make_float4(0.f, 0.f, 0.f, 0.f), rq = ev;
            float2 cv = make_float2(0.f, 0.f);
            if (inside && zA >= 0 && zA < g.nz) {
                ev = cvt4r<VT>(*reinterpret_cast<const R4*>(&S.ev[k][0][0] + vo));
                rq = cvt4r<VT>(*reinterpret_cast<const R4*>(&S.rv[k][0][0] + vo));
                cv = cvt2(*reinterpret_cast<const C2*>(&S.ec[k >> 1][0] + co));
            }
            const int p = par ^ (k & 1);
            const float2 er = p ? make_float2(ev.y, ev.w) : make_float2(ev.x, ev.z);
            const float2 rb = p ? make_float2(rq.x, rq.z) : make_float2(rq.y, rq.w);
            float* EP = e0 + k * SL;
            *reinterpret_cast<float2*>(EP + o + p * HW) = make_float2(fmaf(w, cv.x, er.x), fmaf(w, cv.y, er.y));
            *reinterpret_cast<float2*>(EP + o + (1 - p) * HW) = make_float2(1.0f * rb.x, 1.0f * rb.y);
        }
    }
    __syncthreads();
    // ---- black half-step, planes 1 .. np-2 over the 1-halo rows, in place
    if (ok && t < G::NBLK) {
        int row, q;
        stage_task(t, G::NBR, 1, &row, &q);
        const int ob = row * RW + 2 * q;
        const int par = (y0 - 2 + row) & 1;
#pragma unroll
        for (int k = 1; k < NP - 1; k++) {
            if (k > np - 2) break;
            const int h = par ^ ((k + 1) & 1);
            const int o = ob + h * HW;
            float* E = e0 + k * SL;
            float2 d;
            const float2 s = gs_sum2<CK>(c0 + k * SL, c0 + (k + 1) * SL, E, E - SL, E + SL, o, h,
                                         *reinterpret_cast<const float2*>(E + o), &d);
            *reinterpret_cast<float2*>(E + o) = divide2(s, d);
        }
    }
    __syncthreads();
    // ---- red half-step, planes 2 .. np-3 over the tile, out = z
    if (ok && t < G::NOWN) {
        const int tx = t % QX, ty = t / QX;
        const int ox = x0 + 4 * tx, oy = y0 + ty;
        const bool own_inside = ox < g.nx && oy < g.ny;
        const int oo = (ty + 2) * RW + 2 * (tx + 1);
        const int ov = (ty + 2) * V::VW + V::VX + 4 * (tx + 1);
        const long long og = ox + (long long)g.nx * oy;
        for (int k = 2; k < np - 2; k++) {
            const int zC = zs + k;
            const float* E = e0 + k * SL;
            const int p = (oy & 1) ^ (k & 1);
            const float4 rv = cvt4r<VT>(*reinterpret_cast<const R4*>(&S.rv[k][0][0] + ov));
            const float2 rr = p ? make_float2(rv.y, rv.w) : make_float2(rv.x, rv.z);
            float2 d;
            const float2 s = gs_sum2<CK>(c0 + k * SL, c0 + (k + 1) * SL, E, E - SL, E + SL, oo + p * HW, p,
                                         make_float2(1.0f * rr.x, 1.0f * rr.y), &d);
            const float2 zr = divide2(s, d);
            const float2 zb = *reinterpret_cast<const float2*>(E + oo + (1 - p) * HW);
            float4 zv = p ? make_float4(zb.x, zr.x, zb.y, zr.y) : make_float4(zr.x, zb.x, zr.y, zb.y);
            if (own_inside) {
                if (accum) {  // out = accum + z (second W-cycle visit)
                    const float4 a = cvt4r<VT>(*reinterpret_cast<const R4*>(accum + og + sxy * zC));
                    zv = make_float4(a.x + zv.x, a.y + zv.y, a.z + zv.z, a.w + zv.w);
                }
                st4<VT>(out + og + sxy * zC, zv);
            }
        }
    }
    run_drain(S, np, ISSUER);
}

// ------------------------------------------------------------------ host
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
bool g_tma_enabled = false;
int g_sms = 0;
int g_occ[3][2][2] = {};  // [records precision][coarse level][pre / post]: resident blocks per SM

bool encoder() {
    static std::once_flag once;
    std::call_once(once, [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
        else
            (void)cudaGetLastError();
    });
    return g_encode != nullptr;
}

// 3-D map of a level vector (x-fastest cells, element size 4 or 2 bytes),
// box w x rows x 1.
bool vec_map(CUtensorMap* m, const void* base, int esize, const Grid3& g, int w, int rows) {
    const cuuint64_t dims[3] = {(cuuint64_t)g.nx, (cuuint64_t)g.ny, (cuuint64_t)g.nz};
    const cuuint64_t strides[2] = {(cuuint64_t)g.nx * esize, (cuuint64_t)g.nx * g.ny * esize};
    const cuuint32_t box[3] = {(cuuint32_t)w, (cuuint32_t)rows, 1};
    const cuuint32_t es[3] = {1, 1, 1};
    return g_encode(m, esize == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_UINT16, 3,
                    const_cast<void*>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
// 4-D map of the split-row smoother records: (4 values x nx/2 records of a
// half row, even/odd half, y, z), box 144 values x 2 halves x rows x 1.
bool rec_map(CUtensorMap* m, const void* base, int ck, const Grid3& g, int rows) {
    const int esize = ck == 0 ? 4 : 2;
    const cuuint64_t half = (cuuint64_t)2 * g.nx;  // values per half row
    const cuuint64_t dims[4] = {half, 2, (cuuint64_t)g.ny, (cuuint64_t)g.nz};
    const cuuint64_t strides[3] = {half * esize, 2 * half * esize, 2 * half * esize * g.ny};
    const cuuint32_t box[4] = {(cuuint32_t)(2 * RW), 2, (cuuint32_t)rows, 1};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    return g_encode(m, esize == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_UINT16, 4,
                    const_cast<void*>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// z runs as in fused_launch: even runs that fill whole waves of resident
// blocks, each run computing two planes below and above it.
Launch tma_launch(const Grid3& g0, int fty, int nt, int occ) {
    Launch P;
    P.g = g0;
    P.block = dim3(nt, 1, 1);
    const int gx = (g0.nx + PX - 1) / PX, gy = (g0.ny + fty - 1) / fty, nz = g0.nz;
    const int tiles = gx * gy;
    const int cap = (g_sms > 0 ? g_sms : 152) * (occ > 0 ? occ : 1);
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

template <int CK, class VT, class VTc, bool UPDATE, bool FINE>
bool pre_tma(const Grid3& g, const Grid3& gc, const void* sm, const void* rin, const float* q, float* r_out, void* e,
             void* rc, Scalars* sc, double* partials, cudaStream_t s) {
    using G = TGeo<CK>;
    if (!aligned16(sm) || !aligned16(rin) || (UPDATE && !aligned16(q))) return false;
    CUtensorMap tm_rec, tm_r, tm_q;
    if (!rec_map(&tm_rec, sm, CK, g, G::RH)) return false;
    if (!vec_map(&tm_r, rin, (int)sizeof(VT), g, VGeo<VT>::VW, G::RH)) return false;
    if (UPDATE) {
        if (!vec_map(&tm_q, q, 4, g, VGeo<float>::VW, G::RH)) return false;
    } else {
        tm_q = tm_r;
    }
    const Launch P = tma_launch(g, G::FTY, G::NT, g_occ[CK][FINE ? 0 : 1][0]);
    k_pre_tma<CK, VT, VTc, UPDATE, FINE><<<P.grid, P.block, sizeof(PreTmaSm<CK, VT, UPDATE>) + 128, s>>>(
        tm_rec, tm_r, tm_q, P.g, gc, r_out, (VT*)e, (VTc*)rc, sc, partials, P.nblocks);
    return true;
}
template <int CK, class VT, class VTc, bool DOT, bool FINE>
bool post_tma(const Grid3& g, const Grid3& gc, const void* sm, const void* e, const void* ec, const void* r, void* out,
              const void* accum, float w, Scalars* sc, double* partials, long long n_active, cudaStream_t s) {
    using G = TGeo<CK>;
    if (!aligned16(sm) || !aligned16(e) || !aligned16(r) || !aligned16(ec)) return false;
    if ((gc.nx * (int)sizeof(VTc)) % 16) return false;
    CUtensorMap tm_rec, tm_e, tm_r, tm_ec;
    if (!rec_map(&tm_rec, sm, CK, g, G::RH)) return false;
    if (!vec_map(&tm_e, e, (int)sizeof(VT), g, VGeo<VT>::VW, G::RH)) return false;
    if (!vec_map(&tm_r, r, (int)sizeof(VT), g, VGeo<VT>::VW, G::RH)) return false;
    if (!vec_map(&tm_ec, ec, (int)sizeof(VTc), gc, G::CW, G::CRH)) return false;
    const Launch P = tma_launch(g, G::FTY, G::NT, g_occ[CK][FINE ? 0 : 1][1]);
    k_post_tma<CK, VT, VTc, DOT, FINE><<<P.grid, P.block, sizeof(PostTmaSm<CK, VT, VTc>) + 128, s>>>(
        tm_rec, tm_e, tm_r, tm_ec, P.g, (VT*)out, (const VT*)accum, w, sc, partials, P.nblocks, n_active);
    return true;
}

// Coarse levels whose runs of two planes fill at most one wave of one block
// per SM take the whole-run passes.
bool whole_runs(const Grid3& g, int fty) {
    const long long tiles = (long long)((g.nx + PX - 1) / PX) * ((g.ny + fty - 1) / fty);
    return tiles * ((g.nz + 1) / 2) <= (g_sms > 0 ? g_sms : 152);
}
template <int CK, class VT, class VTc>
bool pre_run(const Grid3& g, const Grid3& gc, const void* sm, const void* rin, void* e, void* rc, Scalars* sc,
             cudaStream_t s) {
    using G = TGeo<CK>;
    if (!aligned16(sm) || !aligned16(rin)) return false;
    CUtensorMap tm_rec, tm_r;
    if (!rec_map(&tm_rec, sm, CK, g, G::RH)) return false;
    if (!vec_map(&tm_r, rin, (int)sizeof(VT), g, VGeo<VT>::VW, G::RH)) return false;
    const dim3 grid((g.nx + PX - 1) / PX, (g.ny + G::FTY - 1) / G::FTY, (g.nz + 1) / 2);
    k_pre_run<CK, VT, VTc><<<grid, G::NT, sizeof(PreRunSm<CK, VT>) + 128, s>>>(tm_rec, tm_r, g, gc, (VT*)e,
                                                                              (VTc*)rc, sc);
    return true;
}
template <int CK, class VT, class VTc>
bool post_run(const Grid3& g, const Grid3& gc, const void* sm, const void* e, const void* ec, const void* r, void* out,
              const void* accum, float w, Scalars* sc, cudaStream_t s) {
    using G = TGeo<CK>;
    if (!aligned16(sm) || !aligned16(e) || !aligned16(r) || !aligned16(ec)) return false;
    if ((gc.nx * (int)sizeof(VTc)) % 16) return false;
    CUtensorMap tm_rec, tm_e, tm_r, tm_ec;
    if (!rec_map(&tm_rec, sm, CK, g, G::RH)) return false;
    if (!vec_map(&tm_e, e, (int)sizeof(VT), g, VGeo<VT>::VW, G::RH)) return false;
    if (!vec_map(&tm_r, r, (int)sizeof(VT), g, VGeo<VT>::VW, G::RH)) return false;
    if (!vec_map(&tm_ec, ec, (int)sizeof(VTc), gc, G::CW, G::CRH)) return false;
    const dim3 grid((g.nx + PX - 1) / PX, (g.ny + G::FTY - 1) / G::FTY, (g.nz + 1) / 2);
    k_post_run<CK, VT, VTc><<<grid, G::NT, sizeof(PostRunSm<CK, VT, VTc>) + 128, s>>>(
        tm_rec, tm_e, tm_r, tm_ec, g, (VT*)out, (const VT*)accum, w, sc);
    return true;
}

template <class F>
cudaError_t prep(F* fn, size_t bytes, int threads, int* occ) {
    cudaError_t e = cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess && occ) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, (const void*)fn, threads, bytes);
    return e;
}
template <int CK, class VT, class VTc>
cudaError_t prep_level(bool fine) {
    using G = TGeo<CK>;
    cudaError_t e = cudaSuccess;
    const size_t pre_u = sizeof(PreTmaSm<CK, VT, true>) + 128, pre_n = sizeof(PreTmaSm<CK, VT, false>) + 128;
    const size_t post = sizeof(PostTmaSm<CK, VT, VTc>) + 128;
    if (fine) {
        if (e == cudaSuccess) e = prep(k_pre_tma<CK, VT, VTc, true, true>, pre_u, G::NT, &g_occ[CK][0][0]);
        if (e == cudaSuccess) e = prep(k_pre_tma<CK, VT, VTc, false, true>, pre_n, G::NT, nullptr);
        if (e == cudaSuccess) e = prep(k_post_tma<CK, VT, VTc, true, true>, post, G::NT, &g_occ[CK][0][1]);
    } else {
        if (e == cudaSuccess) e = prep(k_pre_tma<CK, VT, VTc, false, false>, pre_n, G::NT, &g_occ[CK][1][0]);
        if (e == cudaSuccess) e = prep(k_post_tma<CK, VT, VTc, false, false>, post, G::NT, &g_occ[CK][1][1]);
        if (e == cudaSuccess) e = prep(k_pre_run<CK, VT, VTc>, sizeof(PreRunSm<CK, VT>) + 128, G::NT, nullptr);
        if (e == cudaSuccess)
            e = prep(k_post_run<CK, VT, VTc>, sizeof(PostRunSm<CK, VT, VTc>) + 128, G::NT, nullptr);
    }
    return e;
}
}  // namespace

bool tma_fused_enabled() { return g_tma_enabled; }

cudaError_t tma_prepare_attributes() {
    const char* ev = getenv("MHDPROJ_TMA");
    g_tma_enabled = !(ev && ev[0] == '0') && encoder();
    if (!g_tma_enabled) return cudaSuccess;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = prep_level<0, float, float>(true);
    if (e == cudaSuccess) e = prep_level<1, float, __half>(true);
    if (e == cudaSuccess) e = prep_level<2, float, __nv_bfloat16>(true);
    if (e == cudaSuccess) e = prep_level<0, float, float>(false);
    if (e == cudaSuccess) e = prep_level<1, __half, __half>(false);
    if (e == cudaSuccess) e = prep_level<2, __nv_bfloat16, __nv_bfloat16>(false);
    return e;
}

static bool tma_grid_ok(const Grid3& g, int vt_bytes) {
    return g_tma_enabled && g.periodic == 0 && g.nx % 4 == 0 && (g.nx * vt_bytes) % 16 == 0;
}

bool tma_pre(int ck, bool fine, bool update, const Grid3& g, const Grid3& gc, const void* sm, const void* rin,
             const float* q, float* r_out, void* e, void* rc, Scalars* sc, double* partials, cudaStream_t s) {
    const int vt = fine || ck == 0 ? 4 : 2;
    if (!tma_grid_ok(g, vt)) return false;
    if (fine) {
        if (ck == 1)
            return update ? pre_tma<1, float, __half, true, true>(g, gc, sm, rin, q, r_out, e, rc, sc, partials, s)
                          : pre_tma<1, float, __half, false, true>(g, gc, sm, rin, q, r_out, e, rc, sc, partials, s);
        if (ck == 2)
            return update
                       ? pre_tma<2, float, __nv_bfloat16, true, true>(g, gc, sm, rin, q, r_out, e, rc, sc, partials, s)
                       : pre_tma<2, float, __nv_bfloat16, false, true>(g, gc, sm, rin, q, r_out, e, rc, sc, partials, s);
        return update ? pre_tma<0, float, float, true, true>(g, gc, sm, rin, q, r_out, e, rc, sc, partials, s)
                      : pre_tma<0, float, float, false, true>(g, gc, sm, rin, q, r_out, e, rc, sc, partials, s);
    }
    if (whole_runs(g, ck == 0 ? TGeo<0>::FTY : TGeo<1>::FTY)) {
        if (ck == 1) return pre_run<1, __half, __half>(g, gc, sm, rin, e, rc, sc, s);
        if (ck == 2) return pre_run<2, __nv_bfloat16, __nv_bfloat16>(g, gc, sm, rin, e, rc, sc, s);
        return pre_run<0, float, float>(g, gc, sm, rin, e, rc, sc, s);
    }
    if (ck == 1) return pre_tma<1, __half, __half, false, false>(g, gc, sm, rin, q, r_out, e, rc, sc, partials, s);
    if (ck == 2)
        return pre_tma<2, __nv_bfloat16, __nv_bfloat16, false, false>(g, gc, sm, rin, q, r_out, e, rc, sc, partials, s);
    return pre_tma<0, float, float, false, false>(g, gc, sm, rin, q, r_out, e, rc, sc, partials, s);
}

bool tma_post(int ck, bool fine, const Grid3& g, const Grid3& gc, const void* sm, const void* e, const void* ec,
              const void* r, void* out, const void* accum, float w, Scalars* sc, double* partials, long long n_active,
              cudaStream_t s) {
    const int vt = fine || ck == 0 ? 4 : 2;
    if (!tma_grid_ok(g, vt)) return false;
    if (fine) {
        if (ck == 1)
            return post_tma<1, float, __half, true, true>(g, gc, sm, e, ec, r, out, accum, w, sc, partials, n_active, s);
        if (ck == 2)
            return post_tma<2, float, __nv_bfloat16, true, true>(g, gc, sm, e, ec, r, out, accum, w, sc, partials,
                                                                 n_active, s);
        return post_tma<0, float, float, true, true>(g, gc, sm, e, ec, r, out, accum, w, sc, partials, n_active, s);
    }
    if (whole_runs(g, ck == 0 ? TGeo<0>::FTY : TGeo<1>::FTY)) {
        if (ck == 1) return post_run<1, __half, __half>(g, gc, sm, e, ec, r, out, accum, w, sc, s);
        if (ck == 2) return post_run<2, __nv_bfloat16, __nv_bfloat16>(g, gc, sm, e, ec, r, out, accum, w, sc, s);
        return post_run<0, float, float>(g, gc, sm, e, ec, r, out, accum, w, sc, s);
    }
    if (ck == 1)
        return post_tma<1, __half, __half, false, false>(g, gc, sm, e, ec, r, out, accum, w, sc, partials, n_active, s);
    if (ck == 2)
        return post_tma<2, __nv_bfloat16, __nv_bfloat16, false, false>(g, gc, sm, e, ec, r, out, accum, w, sc,
                                                                       partials, n_active, s);
    return post_tma<0, float, float, false, false>(g, gc, sm, e, ec, r, out, accum, w, sc, partials, n_active, s);
}

}  // namespace mhdproj
