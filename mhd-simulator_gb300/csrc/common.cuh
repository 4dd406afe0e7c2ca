// common.cuh -- shared device helpers for the GB300 projection kernels.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>

namespace mhdproj {

// Tiles: 32 x 8 threads over (x, y); each thread walks a run of z.
constexpr int TX = 32;
constexpr int TY = 8;
constexpr int TILE_THREADS = TX * TY;
// Upper bound on blocks of a reduction launch (the partials arrays are sized by it).
constexpr int MAX_REDUCE_BLOCKS = 8192;

struct Grid3 {
    int nx, ny, nz;
    int periodic;  // bit a: axis a periodic
    int zper;      // z cells per block (tile launches)
    __host__ __device__ long long n() const { return (long long)nx * ny * nz; }
};

// Device scalar block of the CG solver.  Written only by last-block
// reductions (single writer) and read by every kernel of the iteration.
struct Scalars {
    double bb;          // ||b||^2 (FP64)
    double rr_true;     // ||b - A phi||^2 of the last refinement residual
    double rr;          // inner ||r||^2
    double rr_target;   // inner stop threshold on ||r||^2
    double rz;          // r . z (preconditioned)
    double pq;          // p . A p
    double alpha, beta; // CG scalars
    double abs_floor;   // absolute floor on ||r||^2 (reference abs_div_tol term)
    double tol2;        // relative tolerance squared
    double inner_floor2;// minimum inner relative reduction squared
    double objective;   // chain objective / misc reductions
    double divmax, div2;// divergence statistics
    float alpha_f, beta_f, sigma, inv_sigma;
    float inv_sigma_z;  // 1/sigma of the V-cycle that produced the current z
    int first;          // the next search step starts a CG pass (p = z, no x update)
    int pidx;           // search-direction buffer written last (pipelined CG)
    int max_total;      // iteration cap checked on the device (pipelined CG)
    int converged;      // inner solve finished
    int outer_done;     // true residual meets the target
    int iterations;     // inner iterations of this solve
    int total_iterations;
    int nonfinite;      // a reduction produced NaN/Inf
    int breakdown;      // p.Ap <= 0
    int stalled;        // a bounded device-side wait ran out (the solve stops)
    unsigned int ticket[12];
};

// ------------------------------------------------------------ indexing
__device__ __forceinline__ int wrap_or_neg(int c, int n, bool periodic) {
    if (c < 0) return periodic ? c + n : -1;
    if (c >= n) return periodic ? c - n : -1;
    return c;
}

// A thread's (x, y) column for kernels that march along z: neighbour offsets
// are computed once; an absent neighbour (closed boundary) gets offset 0 so
// every load stays in bounds, and its coefficient is zero by construction.
struct Column {
    int i0, sxy, nz;
    int dxm, dxp, dym, dyp;
    bool hxp, hyp, pz;
    __device__ __forceinline__ Column(const Grid3& g, int x, int y) {
        sxy = g.nx * g.ny;
        nz = g.nz;
        i0 = x + g.nx * y;
        const bool px = g.periodic & 1, py = g.periodic & 2;
        pz = (g.periodic & 4) != 0;
        dxm = x > 0 ? -1 : (px ? g.nx - 1 : 0);
        dxp = x + 1 < g.nx ? 1 : (px ? -(g.nx - 1) : 0);
        hxp = x + 1 < g.nx || px;
        dym = y > 0 ? -g.nx : (py ? g.nx * (g.ny - 1) : 0);
        dyp = y + 1 < g.ny ? g.nx : (py ? -g.nx * (g.ny - 1) : 0);
        hyp = y + 1 < g.ny || py;
    }
    __device__ __forceinline__ int at(int z) const { return i0 + z * sxy; }
    __device__ __forceinline__ bool zexists(int z) const { return pz || (z >= 0 && z < nz); }
    // index of plane z (wrapped when periodic, clamped otherwise)
    __device__ __forceinline__ int zat(int z) const {
        int w = z;
        if (w < 0) w = pz ? w + nz : 0;
        else if (w >= nz) w = pz ? w - nz : nz - 1;
        return at(w);
    }
};

// ------------------------------------------------ rounding-explicit FP32
// The mobility is computed with an operation order shared with the CPU
// oracle; explicit intrinsics stop the compiler from fusing multiply-adds.
__device__ __forceinline__ float rho_of(float a, float rho_l, float rho_air) {
    return __fadd_rn(__fmul_rn(rho_air, __fsub_rn(1.0f, a)), __fmul_rn(rho_l, a));
}
__device__ __forceinline__ float beta_of(float aL, float aR, float rho_l, float rho_air) {
    return __fdiv_rn(rho_l, __fmul_rn(0.5f, __fadd_rn(rho_of(aL, rho_l, rho_air), rho_of(aR, rho_l, rho_air))));
}
__device__ __forceinline__ float outlet_conductance(float a, float rho_l, float rho_air) {
    return __fmul_rn(2.0f, __fdiv_rn(rho_l, rho_of(a, rho_l, rho_air)));
}

// Face mobility of the GB300 solver (mobility, src/fluid/solver.wgsl:43-51):
// beta = rho_l / mean face density with two phases, 1 with one phase
// (SurfaceConfig disabled); with a thermal phase field, divided by
// 1 + dt * drag where drag = rate (1 - f)^2 / (f^3 + 1e-3) and f is the
// smaller phase fraction of the two cells.  Same operation order as the
// reference and the oracle, no fused multiply-adds.
struct Mobility {
    float rho_l, rho_air;
    int single;          // one phase: beta = 1
    const float* phase;  // thermal phase fraction per cell, or nullptr (no drag)
    float drag_rate, dt;
};
__device__ __forceinline__ float mobility_of(const Mobility& m, float aL, float aR, long long iL, long long iR) {
    float b = m.single ? 1.0f : beta_of(aL, aR, m.rho_l, m.rho_air);
    if (m.phase) {
        const float f = fminf(__ldg(m.phase + iL), __ldg(m.phase + iR));
        const float om = __fsub_rn(1.0f, f);
        const float drag = __fdiv_rn(__fmul_rn(__fmul_rn(m.drag_rate, om), om),
                                     __fadd_rn(__fmul_rn(__fmul_rn(f, f), f), 1e-3f));
        b = __fdiv_rn(b, __fadd_rn(1.0f, __fmul_rn(m.dt, drag)));
    }
    return b;
}
// Dirichlet outlet: conductance 2 beta to p = 0 half a cell above the cell
// (beta of the cell with itself; 2 rho_l / rho with two phases).
__device__ __forceinline__ float outlet_mobility(const Mobility& m, float a, long long i) {
    return __fmul_rn(2.0f, mobility_of(m, a, a, i, i));
}

// ------------------------------------------------------ storage types
struct CoefF32 { using store = float4; };
struct CoefF16 { using store = uint2; };
struct CoefBF16 { using store = uint2; };

__device__ __forceinline__ float4 load_coef(const float4* p, long long i) { return __ldg(p + i); }
__device__ __forceinline__ float4 load_coef_h(const uint2* p, long long i) {
    uint2 u = __ldg(p + i);
    __half2 a = *reinterpret_cast<__half2*>(&u.x), b = *reinterpret_cast<__half2*>(&u.y);
    float2 fa = __half22float2(a), fb = __half22float2(b);
    return make_float4(fa.x, fa.y, fb.x, fb.y);
}
__device__ __forceinline__ float4 load_coef_b(const uint2* p, long long i) {
    uint2 u = __ldg(p + i);
    __nv_bfloat162 a = *reinterpret_cast<__nv_bfloat162*>(&u.x), b = *reinterpret_cast<__nv_bfloat162*>(&u.y);
    float2 fa = __bfloat1622float2(a), fb = __bfloat1622float2(b);
    return make_float4(fa.x, fa.y, fb.x, fb.y);
}
__device__ __forceinline__ uint2 pack_coef_h(float4 c) {
    __half2 a = __floats2half2_rn(c.x, c.y), b = __floats2half2_rn(c.z, c.w);
    uint2 u;
    u.x = *reinterpret_cast<unsigned*>(&a);
    u.y = *reinterpret_cast<unsigned*>(&b);
    return u;
}
__device__ __forceinline__ uint2 pack_coef_b(float4 c) {
    __nv_bfloat162 a = __floats2bfloat162_rn(c.x, c.y), b = __floats2bfloat162_rn(c.z, c.w);
    uint2 u;
    u.x = *reinterpret_cast<unsigned*>(&a);
    u.y = *reinterpret_cast<unsigned*>(&b);
    return u;
}

// Scalar vector element types.
__device__ __forceinline__ float to_f(float v) { return v; }
__device__ __forceinline__ float to_f(__half v) { return __half2float(v); }
__device__ __forceinline__ float to_f(__nv_bfloat16 v) { return __bfloat162float(v); }
template <class T> __device__ __forceinline__ T from_f(float v);
template <> __device__ __forceinline__ float from_f<float>(float v) { return v; }
template <> __device__ __forceinline__ __half from_f<__half>(float v) { return __float2half_rn(v); }
template <> __device__ __forceinline__ __nv_bfloat16 from_f<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }

// ------------------------------------------------ double-FP32 arithmetic
// GB300 runs FP64 at a small fraction of its FP32 rate, so values that need
// more than FP32 precision (the refinement residual, the accumulated
// potential, the right-hand side) are carried as unevaluated sums hi + lo of
// two FP32 numbers, with error-free transformations (Knuth's TwoSum, the
// FMA-based TwoProduct; Dekker 1971, Ogita-Rump-Oishi 2005).  That gives
// about 48 significant bits on the FP32 pipes.
struct df {
    float hi, lo;
};
__device__ __forceinline__ df two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
__device__ __forceinline__ df fast_two_sum(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ df df_add(df a, df b) {
    df s = two_sum(a.hi, b.hi);
    const df t = two_sum(a.lo, b.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = fast_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ df df_add_f(df a, float b) {
    df s = two_sum(a.hi, b);
    s.lo = __fadd_rn(s.lo, a.lo);
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_mul_f(df a, float b) {
    df p = two_prod(a.hi, b);
    p.lo = __fmaf_rn(a.lo, b, p.lo);
    return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ float df_to_f(df a) { return __fadd_rn(a.hi, a.lo); }

// Compensated accumulator of FP32 products (Dot2): exact products, TwoSum
// accumulation; the thread total is handed to FP64 only once per thread.
struct Acc {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float x) {
        const df t = two_sum(s, x);
        s = t.hi;
        c = __fadd_rn(c, t.lo);
    }
    __device__ __forceinline__ void add_prod(float a, float b) {
        const df p = two_prod(a, b);
        const df t = two_sum(s, p.hi);
        s = t.hi;
        c = __fadd_rn(c, __fadd_rn(t.lo, p.lo));
    }
    __device__ __forceinline__ double total() const { return (double)s + (double)c; }
};

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

// ------------------------------------------------------- reductions
__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide sum of K doubles (blockDim.x*y*z == 256); the result is valid in
// thread 0.  Uses the caller's shared buffer of 8*K doubles.
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K], double* sh) {
    const int t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int lane = t & 31, warp = t >> 5;
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = warp_sum(v[k]);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; k++) sh[warp * K + k] = v[k];
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x * blockDim.y * blockDim.z) >> 5;
#pragma unroll
        for (int k = 0; k < K; k++) {
            double s = lane < nw ? sh[lane * K + k] : 0.0;
            v[k] = warp_sum(s);
        }
    }
    __syncthreads();
}

// Store this block's K partial sums; returns true in the block that arrives
// last (threadFenceReduction pattern).  `partials` is laid out [K][nblocks].
template <int K>
__device__ __forceinline__ bool store_partials_is_last(const double (&v)[K], double* partials, int nblocks,
                                                       unsigned int* ticket) {
    __shared__ bool last;
    const int t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int b = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    if (t == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) partials[k * nblocks + b] = v[k];
        __threadfence();
        unsigned int arrived = atomicAdd(ticket, 1u);
        last = arrived == (unsigned)(nblocks - 1);
    }
    __syncthreads();
    return last;
}

// In the last block: sum the partials in a fixed order (deterministic), the
// total is returned in thread 0; resets the ticket for the next launch.
template <int K>
__device__ __forceinline__ void finish_partials(double (&tot)[K], const double* partials, int nblocks, double* sh,
                                                unsigned int* ticket) {
    __threadfence();
    const int t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nt = blockDim.x * blockDim.y * blockDim.z;
#pragma unroll
    for (int k = 0; k < K; k++) {
        double s = 0.0;
        for (int b = t; b < nblocks; b += nt) s += ((volatile const double*)partials)[k * nblocks + b];
        tot[k] = s;
    }
    block_sum<K>(tot, sh);
    if (t == 0) *ticket = 0u;
}

}  // namespace mhdproj
