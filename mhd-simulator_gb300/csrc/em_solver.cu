// em_solver.cu -- the implicit EM induction step of the reference
// (EmState::advance_to, src/em/mod.rs:863-1090, on the passes of
// src/em/induction.wgsl) as sm_103a kernels behind the mhdproj_em_* C ABI.
//
// Discretisation (reference): magnetic vector potential on the edges of the
// cell grid, x-edges then y-edges then z-edges, each block x-fastest
// (src/em/common.wgsl:3-6).  One backward-Euler step solves
//   (C^T nu C + G + mu0 sigma h^2/dt) x = b
// for the reaction increment x with Jacobi-preconditioned CG, where C is the
// edge-to-face curl, nu the face reluctivity, G the nodal gauge on
// non-conducting nodes and b the applied-field, history and motional terms
// (induction.wgsl:132-145).  The host sequence -- power-of-two residual
// rescaling, the prediction guard, 32-iteration batches with a status read
// between them, true-residual restarts, acceptance, rollback and the
// prediction history -- follows advance_to.
//
// GB300 layout: every vec4 record of the reference is split into planar FP32
// arrays (applied potential, its history, edge conductivity, diagonal,
// motional EMF, the CG vectors) plus one byte of gauge/stencil flags per edge;
// cell conductivity and permeability and the three face reluctivity grids are
// tabulated once per material update instead of being decoded from material
// ids inside every operator application.  The 32-iteration batch runs as one
// CUDA graph.
//
// Arithmetic: FP32 in the shader's operation order, compiled without fused
// multiply-adds; the workgroup sums are 256-lane trees and the single-block
// reductions accumulate their partials with a stride of 256 before the tree,
// so results are bit-identical to the FP32 restatement of the same shader.
//
// Also here: the nodal gradient correction advance_to switches to after 1024
// Jacobi iterations (src/em/nodal.wgsl), the motional EMF
// (src/em/motion.wgsl) and the source pass that sums the applied potential
// of wire, surface-current and uniform-field elements (src/em/source.wgsl).
// Also the per-body force integrals (src/em/body-stats.wgsl) and the energy
// ledger (src/em/energy.wgsl).  Not built:
// building the elements from the model (src/em/sources.rs, host code the
// caller keeps).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "mhdproj.h"

namespace {

constexpr int kBlock = 256;
constexpr uint32_t kBatch = 32;        // iterations between status reads (mod.rs:952)

struct EmDev {
    uint32_t n[3], cells;
    uint32_t e[3], E;
    uint32_t initial;  // control.y: the applied-field solve has no mass term
    uint32_t nodal;    // control.w: the nodal gradient correction is active
    float pf;          // origin.w: increment prediction factor
    float dt, mu0, h, tol2;
    float origin[3];
    // edges
    float *as, *asp, *sig, *diag, *emf;
    uint8_t* flags;  // bit 0: lower node gauged, bit 1: upper node gauged, bit 2: air stencil
    float *x, *r, *p, *w, *prev;
    // cells and faces
    float *sig_c, *mu_c;
    float* nu[3];
    float* nv;  // (nx+1)(ny+1)(nz+1) nodal corrections
    float4* partials;
    float4* scalars;  // [0] (rz, rr, bb, threshold) [1] (alpha, beta, iterations, status) [2..5] fields [6].x scale
    float4* results;  // cells x 4: (B,|B|) (J,|J|) (F, heat) (applied B, |applied B|)
    const uint32_t* materials;
    const float* props;
    uint32_t n_props;
    uint32_t vacuum;
    uint32_t* err;
};

__device__ __forceinline__ float fmx(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float fmn(float a, float b) { return a < b ? a : b; }

__device__ __forceinline__ void edge_dims(const EmDev& D, int axis, uint32_t d[3]) {
    d[0] = D.n[0] + 1;
    d[1] = D.n[1] + 1;
    d[2] = D.n[2] + 1;
    d[axis] -= 1;
}
__device__ __forceinline__ bool valid3(const int p[3], const uint32_t d[3]) {
    return p[0] >= 0 && p[1] >= 0 && p[2] >= 0 && p[0] < (int)d[0] && p[1] < (int)d[1] && p[2] < (int)d[2];
}
__device__ __forceinline__ uint32_t edge_offset(const EmDev& D, int axis) {
    return axis == 0 ? 0u : axis == 1 ? D.e[0] : D.e[0] + D.e[1];
}
__device__ __forceinline__ void edge_decode(const EmDev& D, uint32_t i, int p[3], int* axis) {
    int a = 0;
    uint32_t q = i;
    if (q >= D.e[0]) {
        a = 1;
        q -= D.e[0];
        if (q >= D.e[1]) {
            a = 2;
            q -= D.e[1];
        }
    }
    uint32_t d[3];
    edge_dims(D, a, d);
    p[0] = (int)(q % d[0]);
    p[1] = (int)((q / d[0]) % d[1]);
    p[2] = (int)(q / (d[0] * d[1]));
    *axis = a;
}
__device__ __forceinline__ bool on_boundary(const EmDev& D, const int p[3], int axis) {
    const int a = (axis + 1) % 3, b = (axis + 2) % 3;
    return p[a] == 0 || (uint32_t)p[a] == D.n[a] || p[b] == 0 || (uint32_t)p[b] == D.n[b];
}

// kind 0: increment x, 1: search direction p, 2: applied A_s, 4: accepted A,
// 3: accepted + increment + applied (the total potential).
template <int KIND>
__device__ __forceinline__ float a_edge(const EmDev& D, int axis, const int p[3]) {
    uint32_t d[3];
    edge_dims(D, axis, d);
    if (!valid3(p, d)) return 0.0f;
    const uint32_t i = edge_offset(D, axis) + (uint32_t)p[0] + d[0] * ((uint32_t)p[1] + d[1] * (uint32_t)p[2]);
    if (KIND == 0) return D.x[i];
    if (KIND == 1) return D.p[i];
    if (KIND == 2) return D.as[i];
    if (KIND == 4) return D.prev[i];
    return D.prev[i] + D.x[i] + D.as[i];
}
__device__ __forceinline__ bool face_valid(const EmDev& D, int axis, const int p[3], uint32_t* idx) {
    uint32_t d[3] = {D.n[0], D.n[1], D.n[2]};
    d[axis] += 1;
    if (!valid3(p, d)) return false;
    *idx = (uint32_t)p[0] + d[0] * ((uint32_t)p[1] + d[1] * (uint32_t)p[2]);
    return true;
}
template <int KIND>
__device__ __forceinline__ float curl_face(const EmDev& D, int axis, const int p[3]) {
    uint32_t fi;
    if (!face_valid(D, axis, p, &fi)) return 0.0f;
    const int a = (axis + 1) % 3, b = (axis + 2) % 3;
    int qa[3] = {p[0], p[1], p[2]}, qb[3] = {p[0], p[1], p[2]};
    qa[a] += 1;
    qb[b] += 1;
    return a_edge<KIND>(D, b, qa) - a_edge<KIND>(D, b, p) - a_edge<KIND>(D, a, qb) + a_edge<KIND>(D, a, p);
}
__device__ __forceinline__ float mass(const EmDev& D, uint32_t i) {
    if (D.initial) return 0.0f;
    return D.mu0 * D.sig[i] * D.h * D.h / D.dt;
}
__device__ __forceinline__ float diagonal(const EmDev& D, uint32_t i) { return fmx(D.diag[i] + mass(D, i), 1e-30f); }
__device__ __forceinline__ float residual_scale(const EmDev& D) {
    const float s = D.scalars[6].x;
    return s > 0.0f ? s : 1.0f;
}
__device__ __forceinline__ bool active(const EmDev& D) { return D.scalars[1].w == 0.0f; }

// ---- the curl-curl + gauge operator, edge axis fixed at compile time ----
// adjoint_s is the shader's adjoint (induction.wgsl:57-63: the transposed
// curl of nu-weighted face curls) and gauge_s its gauge (:75-80: nodal
// divergences at gauged end nodes), term for term in the shader's order.
// With the axis a template parameter every neighbour offset is a constant
// and positions stay in registers (a runtime axis keeps small position
// arrays in local memory); each kind of potential is read from its array.
template <int K>
__device__ __forceinline__ void bump(int& x, int& y, int& z, int s) {
    if (K == 0) x += s;
    else if (K == 1) y += s;
    else z += s;
}
template <int K>
__device__ __forceinline__ int coord(int x, int y, int z) { return K == 0 ? x : K == 1 ? y : z; }
template <int AX>
__device__ __forceinline__ float edge_at(const EmDev& D, const float* __restrict__ v, int x, int y, int z) {
    const int dx = (int)D.n[0] + (AX != 0), dy = (int)D.n[1] + (AX != 1), dz = (int)D.n[2] + (AX != 2);
    if (x < 0 || y < 0 || z < 0 || x >= dx || y >= dy || z >= dz) return 0.0f;
    const uint32_t off = AX == 0 ? 0u : AX == 1 ? D.e[0] : D.e[0] + D.e[1];
    return v[off + (uint32_t)x + (uint32_t)dx * ((uint32_t)y + (uint32_t)dy * (uint32_t)z)];
}
template <int F>
__device__ __forceinline__ bool face_at(const EmDev& D, int x, int y, int z, uint32_t* idx) {
    const int fx = (int)D.n[0] + (F == 0), fy = (int)D.n[1] + (F == 1), fz = (int)D.n[2] + (F == 2);
    if (x < 0 || y < 0 || z < 0 || x >= fx || y >= fy || z >= fz) return false;
    *idx = (uint32_t)x + (uint32_t)fx * ((uint32_t)y + (uint32_t)fy * (uint32_t)z);
    return true;
}
template <int F, bool CONTRAST>
__device__ __forceinline__ float face_s(const EmDev& D, const float* __restrict__ v, int x, int y, int z) {
    uint32_t fi;
    if (!face_at<F>(D, x, y, z, &fi)) return 0.0f;
    constexpr int A = (F + 1) % 3, B = (F + 2) % 3;
    float nu = D.nu[F][fi];
    if (CONTRAST) nu = 1.0f - nu;
    int ax = x, ay = y, az = z, bx = x, by = y, bz = z;
    bump<A>(ax, ay, az, 1);
    bump<B>(bx, by, bz, 1);
    const float curl = edge_at<B>(D, v, ax, ay, az) - edge_at<B>(D, v, x, y, z) - edge_at<A>(D, v, bx, by, bz) +
                       edge_at<A>(D, v, x, y, z);
    return nu * curl;
}
template <int W, bool CONTRAST>
__device__ __forceinline__ float adjoint_s(const EmDev& D, const float* __restrict__ v, int x, int y, int z) {
    constexpr int A = (W + 1) % 3, B = (W + 2) % 3;
    int ax = x, ay = y, az = z, bx = x, by = y, bz = z;
    bump<A>(ax, ay, az, -1);
    bump<B>(bx, by, bz, -1);
    return face_s<B, CONTRAST>(D, v, x, y, z) - face_s<B, CONTRAST>(D, v, ax, ay, az) -
           face_s<A, CONTRAST>(D, v, x, y, z) + face_s<A, CONTRAST>(D, v, bx, by, bz);
}
__device__ __forceinline__ float node_div_s(const EmDev& D, const float* __restrict__ v, int x, int y, int z) {
    float value = 0.0f;
    value += edge_at<0>(D, v, x, y, z) - edge_at<0>(D, v, x - 1, y, z);
    value += edge_at<1>(D, v, x, y, z) - edge_at<1>(D, v, x, y - 1, z);
    value += edge_at<2>(D, v, x, y, z) - edge_at<2>(D, v, x, y, z - 1);
    return value;
}
template <int W>
__device__ __forceinline__ float gauge_s(const EmDev& D, const float* __restrict__ v, uint8_t f, int x, int y, int z) {
    float value = 0.0f;
    if (f & 1) value += node_div_s(D, v, x, y, z);
    if (f & 2) {
        int ux = x, uy = y, uz = z;
        bump<W>(ux, uy, uz, 1);
        value -= node_div_s(D, v, ux, uy, uz);
    }
    return value;
}
template <int W>
__device__ __forceinline__ void decode_s(const EmDev& D, uint32_t q, int& x, int& y, int& z) {
    const uint32_t dx = D.n[0] + (W != 0), dy = D.n[1] + (W != 1);
    x = (int)(q % dx);
    y = (int)((q / dx) % dy);
    z = (int)(q / (dx * dy));
}
template <int W>
__device__ __forceinline__ bool boundary_s(const EmDev& D, int x, int y, int z) {
    constexpr int A = (W + 1) % 3, B = (W + 2) % 3;
    const int pa = coord<A>(x, y, z), pb = coord<B>(x, y, z);
    return pa == 0 || pa == (int)D.n[A] || pb == 0 || pb == (int)D.n[B];
}
// One edge of each pass with its axis W and its index q inside the axis
// block (k_em_prepare, k_em_apply, k_em_true_residual dispatch on the axis).
template <int W>
__device__ __forceinline__ float2 prepare_edge(const EmDev& D, uint32_t i, uint32_t q) {
    int x, y, z;
    decode_s<W>(D, q, x, y, z);
    if (boundary_s<W>(D, x, y, z)) return make_float2(0.0f, 0.0f);
    const float m = mass(D, i);
    const uint8_t f = D.flags[i];
    const float b = m * D.dt * D.emf[i] - m * (D.as[i] - D.asp[i]) + adjoint_s<W, true>(D, D.as, x, y, z) -
                    adjoint_s<W, false>(D, D.prev, x, y, z) - gauge_s<W>(D, D.prev, f, x, y, z);
    float r = b;
    if (D.pf > 0.0f) r -= adjoint_s<W, false>(D, D.x, x, y, z) + gauge_s<W>(D, D.x, f, x, y, z) + m * D.x[i];
    return make_float2(b, r);
}
template <int W>
__device__ __forceinline__ float apply_edge(const EmDev& D, uint32_t i, uint32_t q) {
    int x, y, z;
    decode_s<W>(D, q, x, y, z);
    const float pv = D.p[i];
    if (boundary_s<W>(D, x, y, z)) return pv;
    return adjoint_s<W, false>(D, D.p, x, y, z) + gauge_s<W>(D, D.p, D.flags[i], x, y, z) + mass(D, i) * pv;
}
template <int W>
__device__ __forceinline__ float true_residual_edge(const EmDev& D, uint32_t i, uint32_t q) {
    int x, y, z;
    decode_s<W>(D, q, x, y, z);
    if (boundary_s<W>(D, x, y, z)) return 0.0f;
    const float m = mass(D, i);
    const uint8_t f = D.flags[i];
    return m * D.dt * D.emf[i] - m * (D.x[i] + (D.as[i] - D.asp[i])) + adjoint_s<W, true>(D, D.as, x, y, z) -
           adjoint_s<W, false>(D, D.prev, x, y, z) - gauge_s<W>(D, D.prev, f, x, y, z) -
           adjoint_s<W, false>(D, D.x, x, y, z) - gauge_s<W>(D, D.x, f, x, y, z);
}
#define EM_BY_AXIS(FN, D, i)                                                         \
    ((i) < (D).e[0]             ? FN<0>((D), (i), (i))                              \
     : (i) < (D).e[0] + (D).e[1] ? FN<1>((D), (i), (i) - (D).e[0])                  \
                                 : FN<2>((D), (i), (i) - (D).e[0] - (D).e[1]))

__device__ __forceinline__ float4 add4(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ float4 coef4(float4 a, float4 b) {
    return make_float4(a.x + b.x, fmn(a.y, b.y), fmx(a.z, b.z), a.w + b.w);
}
__device__ __forceinline__ float4 max4(float4 a, float4 b) {
    return make_float4(fmx(a.x, b.x), fmx(a.y, b.y), fmx(a.z, b.z), fmx(a.w, b.w));
}
__device__ __forceinline__ float4 cmix4(float4 a, float4 b) {
    return make_float4(fmx(a.x, b.x), fmx(a.y, b.y), fmx(a.z, b.z), a.w + b.w);
}

// 256-lane tree in the shader's pairing (lane l absorbs lane l+s for
// s = 128, 64, ..., 1); the last five levels are warp shuffles with the same
// pairing.  The result is valid in thread 0.
template <int OP>
__device__ __forceinline__ float4 tree256(float4 v) {
    __shared__ float4 red[kBlock];
    const int l = threadIdx.x;
    red[l] = v;
    __syncthreads();
#pragma unroll
    for (int s = kBlock / 2; s >= 32; s >>= 1) {
        if (l < s) red[l] = OP == 0 ? add4(red[l], red[l + s]) : coef4(red[l], red[l + s]);
        __syncthreads();
    }
    float4 w = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (l < 32) {
        w = red[l];
#pragma unroll
        for (int s = 16; s > 0; s >>= 1) {
            float4 o;
            o.x = __shfl_down_sync(0xffffffffu, w.x, s);
            o.y = __shfl_down_sync(0xffffffffu, w.y, s);
            o.z = __shfl_down_sync(0xffffffffu, w.z, s);
            o.w = __shfl_down_sync(0xffffffffu, w.w, s);
            w = OP == 0 ? add4(w, o) : coef4(w, o);
        }
    }
    return w;
}
// Single-block reduce over n partials: lane l accumulates l, l+256, ... from
// `init` in that order (loads issued eight at a time), then the tree.
template <int OP>
__device__ __forceinline__ float4 final_reduce(const float4* partials, uint32_t n, float4 init) {
    float4 v = init;
    uint32_t i = threadIdx.x;
    for (; i + 7 * kBlock < n; i += 8 * kBlock) {
        float4 t[8];
#pragma unroll
        for (int k = 0; k < 8; k++) t[k] = partials[i + k * kBlock];
#pragma unroll
        for (int k = 0; k < 8; k++) v = OP == 0 ? add4(v, t[k]) : coef4(v, t[k]);
    }
    for (; i < n; i += kBlock) v = OP == 0 ? add4(v, partials[i]) : coef4(v, partials[i]);
    return tree256<OP>(v);
}
__device__ __forceinline__ uint32_t groups_of(uint32_t n) { return (n + kBlock - 1) / kBlock; }

// ------------------------------------------------------------ material tables
__global__ void __launch_bounds__(kBlock) k_em_cells(EmDev D) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= D.cells) return;
    float sig, mu;
    if (D.vacuum) {
        sig = 0.0f;
        mu = 1.0f;
    } else {
        const uint32_t id = D.materials[i];
        if (id == 0) {
            sig = D.props[0];
            mu = D.props[1];
        } else if (id & 0x80000000u) {
            const uint32_t m = id & 255u;
            if (m >= D.n_props) {
                atomicOr(D.err, 1u);
                sig = 0.0f;
                mu = 1.0f;
            } else {
                const float alpha = (float)((id >> 8) & 0x7fffffu) / 8388607.0f;
                sig = alpha * D.props[2 * m];
                mu = D.props[1] * (1.0f - alpha) + D.props[2 * m + 1] * alpha;
            }
        } else if (id >= D.n_props) {
            atomicOr(D.err, 1u);
            sig = 0.0f;
            mu = 1.0f;
        } else {
            sig = D.props[2 * id];
            mu = D.props[2 * id + 1];
        }
    }
    D.sig_c[i] = sig;
    D.mu_c[i] = mu;
}
__device__ __forceinline__ float cell_mu(const EmDev& D, const int p[3]) {
    const uint32_t d[3] = {D.n[0], D.n[1], D.n[2]};
    if (!valid3(p, d)) return 1.0f;
    return D.mu_c[(uint32_t)p[0] + D.n[0] * ((uint32_t)p[1] + D.n[1] * (uint32_t)p[2])];
}
__device__ __forceinline__ float cell_sig(const EmDev& D, const int p[3]) {
    const uint32_t d[3] = {D.n[0], D.n[1], D.n[2]};
    if (!valid3(p, d)) return 0.0f;
    return D.sig_c[(uint32_t)p[0] + D.n[0] * ((uint32_t)p[1] + D.n[1] * (uint32_t)p[2])];
}
// nu_face (induction.wgsl:32-36): mean of the two cells' reluctivities.
__global__ void __launch_bounds__(kBlock) k_em_faces(EmDev D, int axis, uint32_t count) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= count) return;
    uint32_t d[3] = {D.n[0], D.n[1], D.n[2]};
    d[axis] += 1;
    int p[3] = {(int)(i % d[0]), (int)((i / d[0]) % d[1]), (int)(i / (d[0] * d[1]))};
    int q[3] = {p[0], p[1], p[2]};
    q[axis] -= 1;
    D.nu[axis][i] = 0.5f / cell_mu(D, p) + 0.5f / cell_mu(D, q);
}
__device__ __forceinline__ bool air_node(const EmDev& D, const int p[3]) {
    for (int k = 0; k < 3; k++)
        if (p[k] <= 0 || p[k] >= (int)D.n[k]) return false;
    for (int x = 0; x < 2; x++)
        for (int y = 0; y < 2; y++)
            for (int z = 0; z < 2; z++) {
                const int q[3] = {p[0] - x, p[1] - y, p[2] - z};
                if (cell_sig(D, q) > 0.0f) return false;
            }
    return true;
}
__device__ __forceinline__ float nu_at(const EmDev& D, int axis, const int p[3]) {
    uint32_t fi;
    return face_valid(D, axis, p, &fi) ? D.nu[axis][fi] : 0.0f;
}
// coefficients (induction.wgsl:105-126): edge conductivity, curl diagonal,
// gauge flags, air-stencil eligibility; partials (conducting boundary edges,
// min sigma>0, max sigma, conducting edges).
__global__ void __launch_bounds__(kBlock) k_em_coefficients(EmDev D) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    float4 v = make_float4(0.0f, 1e30f, 0.0f, 0.0f);
    if (i < D.E) {
        int p[3], w;
        edge_decode(D, i, p, &w);
        const int a = (w + 1) % 3, b = (w + 2) % 3;
        float sigma = 0.0f;
        for (int u = 0; u < 2; u++)
            for (int vv = 0; vv < 2; vv++) {
                int q[3] = {p[0], p[1], p[2]};
                q[a] -= u;
                q[b] -= vv;
                sigma += 0.25f * cell_sig(D, q);
            }
        int qa[3] = {p[0], p[1], p[2]}, qb[3] = {p[0], p[1], p[2]};
        qa[a] -= 1;
        qb[b] -= 1;
        const float nb0 = nu_at(D, b, p), nb1 = nu_at(D, b, qa), na0 = nu_at(D, a, p), na1 = nu_at(D, a, qb);
        float diag = nb0 + nb1 + na0 + na1;
        if (on_boundary(D, p, w)) {
            diag = 1.0f;
            if (sigma > 0.0f) v.x = 1.0f;
        }
        int upper[3] = {p[0], p[1], p[2]};
        upper[w] += 1;
        const float lower_air = air_node(D, p) ? 1.0f : 0.0f;
        const float upper_air = air_node(D, upper) ? 1.0f : 0.0f;
        const bool scalar_air =
            lower_air > 0.5f && upper_air > 0.5f && nb0 == 1.0f && nb1 == 1.0f && na0 == 1.0f && na1 == 1.0f;
        D.flags[i] = (uint8_t)((lower_air > 0.5f ? 1 : 0) | (upper_air > 0.5f ? 2 : 0) | (scalar_air ? 4 : 0));
        D.emf[i] = 0.0f;
        D.sig[i] = sigma;
        D.diag[i] = diag + lower_air + upper_air;
        v.y = sigma > 0.0f ? sigma : 1e30f;
        v.z = sigma;
        v.w = sigma > 0.0f ? 1.0f : 0.0f;
    }
    const float4 t = tree256<1>(v);
    if (threadIdx.x == 0) D.partials[blockIdx.x] = t;
}
__global__ void __launch_bounds__(kBlock) k_em_coefficient_check(EmDev D) {
    const float4 t = final_reduce<1>(D.partials, groups_of(D.E), make_float4(0.0f, 1e30f, 0.0f, 0.0f));
    if (threadIdx.x == 0) D.scalars[0] = t;
}

// ------------------------------------------------------------ step passes
// update_sources: the source pass shifts the history (source.wgsl:16-17),
// the initial solve has none; an unchanged field holds (hold_source).
__global__ void __launch_bounds__(kBlock) k_em_sources(EmDev D, const float* applied) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= D.E) return;
    const float old = D.as[i];
    if (applied) {
        const float a = applied[i];
        D.as[i] = a;
        D.asp[i] = D.initial ? a : old;
    } else {
        D.asp[i] = old;
    }
}
// begin_step (induction.wgsl:248-254)
__global__ void __launch_bounds__(kBlock) k_em_begin_step(EmDev D) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i == 0) D.scalars[6].x = 1.0f;
    if (i >= D.E) return;
    const float accepted = D.x[i];
    float guess = 0.0f;
    if (D.pf > 0.0f) {
        int p[3], w;
        edge_decode(D, i, p, &w);
        if (!on_boundary(D, p, w)) guess = D.pf * (accepted - D.prev[i]);
    }
    D.prev[i] = accepted;
    D.x[i] = guess;
}
__global__ void __launch_bounds__(kBlock) k_em_zero_guess(EmDev D) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i < D.E) D.x[i] = 0.0f;
}
__global__ void __launch_bounds__(kBlock) k_em_commit(EmDev D) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i < D.E) D.x[i] += D.prev[i];
}
__global__ void __launch_bounds__(kBlock) k_em_rollback(EmDev D) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= D.E) return;
    D.x[i] = D.prev[i];
    D.as[i] = D.asp[i];
}
// prepare (induction.wgsl:132-147)
__global__ void __launch_bounds__(kBlock) k_em_prepare(EmDev D) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (i < D.E) {
        const float2 br = EM_BY_AXIS(prepare_edge, D, i);
        float b = br.x, r = br.y;
        const float physical_l1 = fabsf(b);
        const float scale = residual_scale(D);
        b /= scale;
        r /= scale;
        const float z = r / diagonal(D, i);
        D.r[i] = r;
        D.p[i] = z;
        D.w[i] = 0.0f;
        v = make_float4(r * z, r * r, b * b, physical_l1);
    }
    const float4 t = tree256<0>(v);
    if (threadIdx.x == 0) D.partials[blockIdx.x] = t;
}
// initial_reduce (induction.wgsl:148-167)
__global__ void __launch_bounds__(kBlock) k_em_initial_reduce(EmDev D) {
    const float4 sum = final_reduce<0>(D.partials, groups_of(D.E), make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    if (threadIdx.x != 0) return;
    const float scale = residual_scale(D);
    float next = scale;
    if (scale == 1.0f && sum.w > 0.0f && (sum.w < 1e-8f || sum.w > 1e8f)) {
        int e = (int)((__float_as_uint(sum.w) >> 23) & 255u) - 127;
        e = e < -100 ? -100 : e > 100 ? 100 : e;
        next = __uint_as_float((uint32_t)(e + 127) << 23);
    }
    float absolute_floor = 1e-38f;
    if (scale != 1.0f) {
        const float floor_norm = 1e-19f / scale;
        absolute_floor = floor_norm * floor_norm;
    }
    const float threshold = sum.z * D.tol2 + absolute_floor;
    D.scalars[6].x = next;
    D.scalars[0] = make_float4(sum.x, sum.y, sum.z, threshold);
    D.scalars[1] = make_float4(next != scale ? next : 0.0f, 0.0f, 0.0f, sum.y <= threshold ? 1.0f : 0.0f);
}
// apply_operator (induction.wgsl:168-190); AIR = 0 forces the full operator.
template <bool AIR>
__global__ void __launch_bounds__(kBlock) k_em_apply(EmDev D) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    float dot = 0.0f;
    if (i < D.E && active(D)) {
        float q;
        if (AIR && (D.flags[i] & 4)) {
            int axis = 0;
            if (i >= D.e[0]) {
                axis = 1;
                if (i >= D.e[0] + D.e[1]) axis = 2;
            }
            uint32_t d[3];
            edge_dims(D, axis, d);
            const uint32_t zs = d[0] * d[1];
            const float c = D.p[i];
            float result = 0.0f;
            result += (c - D.p[i - 1]) + (c - D.p[i + 1]);
            result += (c - D.p[i - d[0]]) + (c - D.p[i + d[0]]);
            result += (c - D.p[i - zs]) + (c - D.p[i + zs]);
            q = result;
        } else {
            q = EM_BY_AXIS(apply_edge, D, i);
        }
        D.w[i] = q;
        dot = D.p[i] * q;
    }
    const float4 t = tree256<0>(make_float4(dot, 0.0f, 0.0f, 0.0f));
    if (threadIdx.x == 0) D.partials[blockIdx.x] = t;
}
__global__ void __launch_bounds__(kBlock) k_em_alpha_reduce(EmDev D) {
    const float4 sum = final_reduce<0>(D.partials, groups_of(D.E), make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    if (threadIdx.x == 0 && D.scalars[1].w == 0.0f) {
        if (sum.x <= 0.0f || fabsf(sum.x) > 3e38f) D.scalars[1].w = 2.0f;
        else D.scalars[1].x = D.scalars[0].x / sum.x;
    }
}
// update_residual (induction.wgsl:197-208)
__global__ void __launch_bounds__(kBlock) k_em_update_residual(EmDev D) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (i < D.E && active(D)) {
        const float alpha = D.scalars[1].x;
        const float r = D.r[i] - alpha * D.w[i];
        const float d = diagonal(D, i);
        D.x[i] = D.x[i] + residual_scale(D) * (alpha * D.p[i]);
        D.r[i] = r;
        D.w[i] = d;
        v = make_float4(r * r / d, r * r, 0.0f, 0.0f);
    }
    const float4 t = tree256<0>(v);
    if (threadIdx.x == 0) D.partials[blockIdx.x] = t;
}
__global__ void __launch_bounds__(kBlock) k_em_beta_reduce(EmDev D) {
    const float4 sum = final_reduce<0>(D.partials, groups_of(D.E), make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    if (threadIdx.x == 0 && D.scalars[1].w == 0.0f) {
        D.scalars[1].y = sum.x / D.scalars[0].x;
        D.scalars[0].x = sum.x;
        D.scalars[0].y = sum.y;
        D.scalars[1].z += 1.0f;
        if (sum.y <= D.scalars[0].w) D.scalars[1].w = 1.0f;
        if (fabsf(sum.x) > 3e38f || fabsf(sum.y) > 3e38f) D.scalars[1].w = 2.0f;
    }
}
// update_search (induction.wgsl:214): z = r/d, or the nodal z left in w
__global__ void __launch_bounds__(kBlock) k_em_update_search(EmDev D) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i < D.E && active(D)) {
        const float z = D.nodal ? D.w[i] : D.r[i] / D.w[i];
        D.p[i] = z + D.scalars[1].y * D.p[i];
    }
}
// true_residual (induction.wgsl:230-240)
__global__ void __launch_bounds__(kBlock) k_em_true_residual(EmDev D) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (i < D.E) {
        float r = EM_BY_AXIS(true_residual_edge, D, i);
        r /= residual_scale(D);
        const float d = diagonal(D, i);
        D.r[i] = r;
        D.p[i] = r / d;
        v = make_float4(r * r / d, r * r, 0.0f, 0.0f);
    }
    const float4 t = tree256<0>(v);
    if (threadIdx.x == 0) D.partials[blockIdx.x] = t;
}
__global__ void __launch_bounds__(kBlock) k_em_restart_reduce(EmDev D) {
    const float4 sum = final_reduce<0>(D.partials, groups_of(D.E), make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    if (threadIdx.x == 0) {
        D.scalars[0].x = sum.x;
        D.scalars[0].y = sum.y;
        D.scalars[1].w = sum.y <= D.scalars[0].w ? 1.0f : 0.0f;
    }
}

// ------------------------------------------------------------ nodal correction
// The additive gradient-space Jacobi correction of src/em/nodal.wgsl: a value
// per interior node from the edge residuals, then z = r/d + nv(lower node)
// - nv(upper node) on every edge.
__device__ __forceinline__ float cached_air_node(const EmDev& D, int x, int y, int z) {
    if (x <= 0 || y <= 0 || z <= 0 || x >= (int)D.n[0] || y >= (int)D.n[1] || z >= (int)D.n[2]) return 0.0f;
    const uint32_t i = (uint32_t)x + D.n[0] * ((uint32_t)y + (D.n[1] + 1) * (uint32_t)z);  // the x-edge at the node
    return (D.flags[i] & 1) ? 1.0f : 0.0f;
}
template <int A>
__device__ __forceinline__ void nodal_axis(const EmDev& D, int x, int y, int z, float& rhs, float& diag) {
    int lx = x, ly = y, lz = z, ux = x, uy = y, uz = z;
    bump<A>(lx, ly, lz, -1);
    bump<A>(ux, uy, uz, 1);
    const uint32_t dx = D.n[0] + (A != 0), dy = D.n[1] + (A != 1);
    const uint32_t off = A == 0 ? 0u : A == 1 ? D.e[0] : D.e[0] + D.e[1];
    const uint32_t out = off + (uint32_t)x + dx * ((uint32_t)y + dy * (uint32_t)z);
    const uint32_t inc = off + (uint32_t)lx + dx * ((uint32_t)ly + dy * (uint32_t)lz);
    rhs += D.r[out] - D.r[inc];
    diag += mass(D, out) + mass(D, inc) + cached_air_node(D, lx, ly, lz) + cached_air_node(D, ux, uy, uz);
}
template <bool INITIAL>
__global__ void __launch_bounds__(kBlock) k_em_nodal_build(EmDev D, uint32_t nodes) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= nodes || (!INITIAL && !active(D))) return;
    const uint32_t d0 = D.n[0] + 1, d1 = D.n[1] + 1;
    const int x = (int)(i % d0), y = (int)((i / d0) % d1), z = (int)(i / (d0 * d1));
    float value = 0.0f;
    if (x > 0 && y > 0 && z > 0 && x < (int)D.n[0] && y < (int)D.n[1] && z < (int)D.n[2]) {
        float rhs = 0.0f, diag = 36.0f * cached_air_node(D, x, y, z);
        nodal_axis<0>(D, x, y, z, rhs, diag);
        nodal_axis<1>(D, x, y, z, rhs, diag);
        nodal_axis<2>(D, x, y, z, rhs, diag);
        value = rhs / fmx(diag, 1e-30f);
    }
    D.nv[i] = value;
}
template <int W>
__device__ __forceinline__ float nodal_z_edge(const EmDev& D, uint32_t i, uint32_t q) {
    int x, y, z;
    decode_s<W>(D, q, x, y, z);
    const uint32_t d0 = D.n[0] + 1, d1 = D.n[1] + 1;
    const uint32_t lo = (uint32_t)x + d0 * ((uint32_t)y + d1 * (uint32_t)z);
    bump<W>(x, y, z, 1);
    const uint32_t up = (uint32_t)x + d0 * ((uint32_t)y + d1 * (uint32_t)z);
    return D.r[i] / diagonal(D, i) + D.nv[lo] - D.nv[up];
}
// nodal_initial / nodal_update: only the x and y lanes of the partials are
// written (the update only while the solve is active).
template <bool INITIAL>
__global__ void __launch_bounds__(kBlock) k_em_nodal(EmDev D) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const bool on = INITIAL || active(D);
    if (i < D.E && on) {
        const float r = D.r[i];
        const float z = EM_BY_AXIS(nodal_z_edge, D, i);
        if (INITIAL) D.p[i] = z;
        D.w[i] = z;
        v = make_float4(r * z, r * r, 0.0f, 0.0f);
    }
    const float4 t = tree256<0>(v);
    if (threadIdx.x == 0 && on) {
        D.partials[blockIdx.x].x = t.x;
        D.partials[blockIdx.x].y = t.y;
    }
}

// ------------------------------------------------------------ fields
__device__ __forceinline__ float electric_edge(const EmDev& D, int axis, const int p[3]) {
    uint32_t d[3];
    edge_dims(D, axis, d);
    if (D.initial || !valid3(p, d)) return 0.0f;
    const uint32_t i = edge_offset(D, axis) + (uint32_t)p[0] + d[0] * ((uint32_t)p[1] + d[1] * (uint32_t)p[2]);
    return -(D.x[i] + (D.as[i] - D.asp[i])) / D.dt + D.emf[i];
}
__device__ __forceinline__ float current_edge(const EmDev& D, int axis, const int p[3]) {
    uint32_t d[3];
    edge_dims(D, axis, d);
    if (!valid3(p, d)) return 0.0f;
    const uint32_t i = edge_offset(D, axis) + (uint32_t)p[0] + d[0] * ((uint32_t)p[1] + d[1] * (uint32_t)p[2]);
    return D.sig[i] * electric_edge(D, axis, p);
}
__device__ __forceinline__ float len3(float x, float y, float z) { return sqrtf(x * x + y * y + z * z); }

// fields (induction.wgsl:188-216): per cell B, J, J x B, Joule heat, applied B
// and the four workgroup reductions (maxima; force and power; div J, max edge
// J, div B, magnetic energy; applied and reaction maxima).
__global__ void __launch_bounds__(kBlock) k_em_fields(EmDev D) {
    __shared__ float4 ra[kBlock], rb[kBlock], rc[kBlock], rd[kBlock];
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    float4 oa = make_float4(0, 0, 0, 0), ob = oa, oc = oa, od = oa;
    if (i < D.cells) {
        const uint32_t nx = D.n[0], ny = D.n[1];
        const int p[3] = {(int)(i % nx), (int)((i / nx) % ny), (int)(i / (nx * ny))};
        const float sig = D.sig_c[i], mu = D.mu_c[i];
        const float h = D.h;
        float mag[3] = {0, 0, 0}, app[3] = {0, 0, 0}, j[3] = {0, 0, 0};
        float heat = 0.0f, div_b = 0.0f, div_j = 0.0f, max_edge = 0.0f, msq = 0.0f;
#pragma unroll
        for (int axis = 0; axis < 3; axis++) {
            int upper[3] = {p[0], p[1], p[2]};
            upper[axis] += 1;
            const float b0 = curl_face<3>(D, axis, p) / h, b1 = curl_face<3>(D, axis, upper) / h;
            msq += 0.5f * (b0 * b0 + b1 * b1);
            mag[axis] = 0.5f * (b0 + b1);
            app[axis] = 0.5f * (curl_face<2>(D, axis, p) + curl_face<2>(D, axis, upper)) / h;
            div_b += b1 - b0;
            const int aa = (axis + 1) % 3, bb = (axis + 2) % 3;
            float es = 0.0f;
            for (int u = 0; u < 2; u++)
                for (int v = 0; v < 2; v++) {
                    int q[3] = {p[0], p[1], p[2]};
                    q[aa] += u;
                    q[bb] += v;
                    const float ee = electric_edge(D, axis, q);
                    es += 0.25f * ee;
                    heat += sig * 0.25f * ee * ee;
                }
            j[axis] = sig * es;
            int prev[3] = {p[0], p[1], p[2]};
            prev[axis] -= 1;
            const float jp = current_edge(D, axis, p), jm = current_edge(D, axis, prev);
            div_j += jp - jm;
            max_edge = fmx(max_edge, fmx(fabsf(jp), fabsf(jm)));
        }
        const float f0 = j[1] * mag[2] - j[2] * mag[1], f1 = j[2] * mag[0] - j[0] * mag[2],
                    f2 = j[0] * mag[1] - j[1] * mag[0];
        const float bn = len3(mag[0], mag[1], mag[2]), jn = len3(j[0], j[1], j[2]), fn = len3(f0, f1, f2);
        const float vol = h * h * h;
        const float an = len3(app[0], app[1], app[2]);
        float4* out = D.results + 4 * (size_t)i;
        out[0] = make_float4(mag[0], mag[1], mag[2], bn);
        out[1] = make_float4(j[0], j[1], j[2], jn);
        out[2] = make_float4(f0, f1, f2, heat);
        out[3] = make_float4(app[0], app[1], app[2], an);
        oa = make_float4(bn, jn, fn, heat);
        ob = make_float4(f0 * vol, f1 * vol, f2 * vol, heat * vol);
        oc = make_float4(fabsf(div_j), max_edge, fabsf(div_b), msq * vol / (2.0f * D.mu0 * mu));
        od = make_float4(an, len3(mag[0] - app[0], mag[1] - app[1], mag[2] - app[2]), 0.0f, 0.0f);
    }
    const int l = threadIdx.x;
    ra[l] = oa;
    rb[l] = ob;
    rc[l] = oc;
    rd[l] = od;
    __syncthreads();
    for (int s = kBlock / 2; s > 0; s >>= 1) {
        if (l < s) {
            ra[l] = max4(ra[l], ra[l + s]);
            rb[l] = add4(rb[l], rb[l + s]);
            rc[l] = cmix4(rc[l], rc[l + s]);
            rd[l] = max4(rd[l], rd[l + s]);
        }
        __syncthreads();
    }
    if (l == 0) {
        float4* P = D.partials + 4 * (size_t)blockIdx.x;
        P[0] = ra[0];
        P[1] = rb[0];
        P[2] = rc[0];
        P[3] = rd[0];
    }
}
__global__ void __launch_bounds__(kBlock) k_em_field_reduce(EmDev D) {
    __shared__ float4 ra[kBlock], rb[kBlock], rc[kBlock], rd[kBlock];
    const uint32_t n = groups_of(D.cells);
    float4 a = make_float4(0, 0, 0, 0), b = a, c = a, d = a;
    for (uint32_t i = threadIdx.x; i < n; i += kBlock) {
        const float4* P = D.partials + 4 * (size_t)i;
        const float4 v = P[2];
        a = max4(a, P[0]);
        b = add4(b, P[1]);
        c = make_float4(fmx(c.x, v.x), fmx(c.y, v.y), fmx(c.z, v.z), c.w + v.w);
        d = max4(d, P[3]);
    }
    const int l = threadIdx.x;
    ra[l] = a;
    rb[l] = b;
    rc[l] = c;
    rd[l] = d;
    __syncthreads();
    for (int s = kBlock / 2; s > 0; s >>= 1) {
        if (l < s) {
            ra[l] = max4(ra[l], ra[l + s]);
            rb[l] = add4(rb[l], rb[l + s]);
            rc[l] = cmix4(rc[l], rc[l + s]);
            rd[l] = max4(rd[l], rd[l + s]);
        }
        __syncthreads();
    }
    if (l == 0) {
        D.scalars[2] = ra[0];
        D.scalars[3] = rb[0];
        D.scalars[4] = rc[0];
        D.scalars[5] = rd[0];
    }
}

// ------------------------------------------------------------ energy ledger
// energy.wgsl after a committed step.  kind 0: new total potential
// (reaction + applied), 1: the previous total, 3: its increment, 2: applied.
template <int KIND>
__device__ __forceinline__ float en_a(const EmDev& D, int axis, const int p[3]) {
    uint32_t d[3];
    edge_dims(D, axis, d);
    if (!valid3(p, d)) return 0.0f;
    const uint32_t i = edge_offset(D, axis) + (uint32_t)p[0] + d[0] * ((uint32_t)p[1] + d[1] * (uint32_t)p[2]);
    if (KIND == 0) return D.x[i] + D.as[i];
    if (KIND == 1) return D.prev[i] + D.asp[i];
    if (KIND == 3) return (D.x[i] - D.prev[i]) + (D.as[i] - D.asp[i]);
    return D.as[i];
}
template <int KIND>
__device__ __forceinline__ float en_curl(const EmDev& D, int axis, const int p[3]) {
    uint32_t fi;
    if (!face_valid(D, axis, p, &fi)) return 0.0f;
    const int a = (axis + 1) % 3, b = (axis + 2) % 3;
    int qa[3] = {p[0], p[1], p[2]}, qb[3] = {p[0], p[1], p[2]};
    qa[a] += 1;
    qb[b] += 1;
    return en_a<KIND>(D, b, qa) - en_a<KIND>(D, b, p) - en_a<KIND>(D, a, qb) + en_a<KIND>(D, a, p);
}
template <int KIND, bool WEIGHTED>
__device__ __forceinline__ float en_face(const EmDev& D, int axis, const int p[3]) {
    uint32_t fi;
    if (!face_valid(D, axis, p, &fi)) return 0.0f;
    return en_curl<KIND>(D, axis, p) * (WEIGHTED ? D.nu[axis][fi] : 1.0f);
}
template <int KIND, bool WEIGHTED>
__device__ __forceinline__ float en_adjoint(const EmDev& D, const int p[3], int w) {
    const int a = (w + 1) % 3, b = (w + 2) % 3;
    int qa[3] = {p[0], p[1], p[2]}, qb[3] = {p[0], p[1], p[2]};
    qa[a] -= 1;
    qb[b] -= 1;
    return en_face<KIND, WEIGHTED>(D, b, p) - en_face<KIND, WEIGHTED>(D, b, qa) -
           en_face<KIND, WEIGHTED>(D, a, p) + en_face<KIND, WEIGHTED>(D, a, qb);
}
__global__ void __launch_bounds__(kBlock) k_em_energy_collect(EmDev D, float4* __restrict__ part) {
    __shared__ float4 ra[kBlock], rb[kBlock];
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    const float h = D.h, dt = D.dt, mu0 = D.mu0, volume = h * h * h;
    float4 a = make_float4(0.0f, 0.0f, 0.0f, 0.0f), b = a;
    if (i < D.E) {
        int p[3], w;
        edge_decode(D, i, p, &w);
        const float delta = (D.x[i] - D.prev[i]) + (D.as[i] - D.asp[i]);
        const float motion = D.emf[i];
        const float ee = -delta / dt + motion;
        const float j = D.sig[i] * ee;
        a.w = dt * volume * j * ee;
        b.x = -dt * volume * j * motion;
        float drive = on_boundary(D, p, w) ? en_adjoint<0, true>(D, p, w) : en_adjoint<2, false>(D, p, w);
        b.y = h / mu0 * delta * drive;
    }
    const uint32_t fx = (D.n[0] + 1) * D.n[1] * D.n[2], fy = D.n[0] * (D.n[1] + 1) * D.n[2],
                   fz = D.n[0] * D.n[1] * (D.n[2] + 1);
    if (i < fx + fy + fz) {
        int axis = 0;
        uint32_t q = i;
        if (q >= fx) {
            q -= fx;
            axis = 1;
            if (q >= fy) {
                q -= fy;
                axis = 2;
            }
        }
        uint32_t d[3] = {D.n[0], D.n[1], D.n[2]};
        d[axis] += 1;
        const int p[3] = {(int)(q % d[0]), (int)((q / d[0]) % d[1]), (int)(q / (d[0] * d[1]))};
        const float now = en_curl<0>(D, axis, p), old = en_curl<1>(D, axis, p), dl = en_curl<3>(D, axis, p);
        const float scale = h / (2.0f * mu0) * D.nu[axis][q];
        a.x = scale * now * now;
        a.y = scale * dl * (now + old);
        a.z = scale * dl * dl;
    }
    const int l = threadIdx.x;
    ra[l] = a;
    rb[l] = b;
    __syncthreads();
    for (int st = kBlock / 2; st > 0; st >>= 1) {
        if (l < st) {
            ra[l] = add4(ra[l], ra[l + st]);
            rb[l] = add4(rb[l], rb[l + st]);
        }
        __syncthreads();
    }
    if (l == 0) {
        part[blockIdx.x] = ra[0];
        part[gridDim.x + blockIdx.x] = rb[0];
    }
}
__global__ void __launch_bounds__(kBlock) k_em_energy_reduce(EmDev D, const float4* __restrict__ part,
                                                              float4* __restrict__ out) {
    const uint32_t n = groups_of(D.E);
    const float4 a = final_reduce<0>(part, n, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    __syncthreads();
    const float4 b = final_reduce<0>(part + n, n, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    if (threadIdx.x == 0) {
        out[0] = a;
        out[1] = b;
    }
}

// ------------------------------------------------------------ body integrals
// body-stats.wgsl: per body z (blockIdx.z) the 256-cell group sums of
// ((fq * h) * h) * h over the cells with bit z set, then one block per body
// reduces its groups.
__global__ void __launch_bounds__(kBlock) k_em_body_collect(EmDev D, const uint32_t* __restrict__ masks,
                                                             float4* __restrict__ part) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    const uint32_t z = blockIdx.z;
    float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (i < D.cells && (masks[i] & (1u << z))) {
        const float4 q = D.results[4 * (size_t)i + 2];
        const float h = D.h;
        v = make_float4(q.x * h * h * h, q.y * h * h * h, q.z * h * h * h, q.w * h * h * h);
    }
    const float4 t = tree256<0>(v);
    if (threadIdx.x == 0) part[(size_t)z * gridDim.x + blockIdx.x] = t;
}
__global__ void __launch_bounds__(kBlock) k_em_body_reduce(EmDev D, const float4* __restrict__ part,
                                                            float4* __restrict__ totals) {
    const uint32_t n = groups_of(D.cells);
    const float4 t = final_reduce<0>(part + (size_t)blockIdx.z * n, n, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    if (threadIdx.x == 0) totals[blockIdx.z] = t;
}

// ------------------------------------------------------------ sources
// The source pass (src/em/source.wgsl:5-17): the applied potential of the
// source elements at every edge midpoint.  Elements arrive in tiles of 32 --
// the reference's batch per pass, whose vector sum is added to the running
// value -- staged in shared memory with the per-element segment direction
// and length; each thread owns one edge.  Kinds (c.y): wire segment a->b
// with core radius c.x and current c.z; surface-current element at a with
// moment b scaled by c.z, softening c.x; uniform field b scaled by c.z.
// Compute-bound: about 60 flops, two logarithms and three square roots per
// wire interaction.
__device__ __forceinline__ float ash(float x) {
    const float sg = x > 0.0f ? 1.0f : x < 0.0f ? -1.0f : 0.0f;
    return sg * logf(fabsf(x) + sqrtf(x * x + 1.0f));
}
constexpr int kTile = 32;
__global__ void __launch_bounds__(kBlock) k_em_source_eval(EmDev D, const float* __restrict__ el, uint32_t count,
                                                            float* __restrict__ out) {
    __shared__ float tile[kTile][14];
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    int w = 0;
    float p[3] = {0.0f, 0.0f, 0.0f};
    if (i < D.E) {
        int e[3];
        edge_decode(D, i, e, &w);
        float pe[3] = {(float)e[0], (float)e[1], (float)e[2]};
        pe[w] += 0.5f;
        p[0] = D.origin[0] + pe[0] * D.h;
        p[1] = D.origin[1] + pe[1] * D.h;
        p[2] = D.origin[2] + pe[2] * D.h;
    }
    float acc = 0.0f;
    const uint32_t nb = count == 0 ? 1u : (count + kTile - 1) / kTile;
    for (uint32_t bi = 0; bi < nb; bi++) {
        __syncthreads();
        if (threadIdx.x < kTile) {
            const uint32_t j = bi * kTile + threadIdx.x;
            float* t = tile[threadIdx.x];
            if (j < count) {
                const float* q = el + 12 * (size_t)j;
                t[0] = q[0];
                t[1] = q[1];
                t[2] = q[2];
                t[3] = q[4];
                t[4] = q[5];
                t[5] = q[6];
                t[6] = q[8];
                t[7] = q[9];
                t[8] = q[10];
                if (q[9] < 0.5f) {
                    const float d0 = q[4] - q[0], d1 = q[5] - q[1], d2 = q[6] - q[2];
                    const float len = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
                    t[9] = d0 / len;
                    t[10] = d1 / len;
                    t[11] = d2 / len;
                    t[12] = len;
                }
            } else {
                t[8] = 0.0f;  // no contribution
            }
        }
        __syncthreads();
        if (i < D.E) {
            const uint32_t left = count - bi * kTile;
            const uint32_t end = count == 0 ? 0u : (left < (uint32_t)kTile ? left : (uint32_t)kTile);
            float a = 0.0f;
            for (uint32_t k = 0; k < end; k++) {
                const float* t = tile[k];
                const float cz = t[8];
                if (cz == 0.0f) continue;
                const float r0 = p[0] - t[0], r1 = p[1] - t[1], r2 = p[2] - t[2];
                const float kind = t[7];
                if (kind < 0.5f) {
                    const float u0 = t[9], u1 = t[10], u2 = t[11], len = t[12];
                    const float tt = r0 * u0 + r1 * u1 + r2 * u2;
                    const float q0 = r0 - u0 * tt, q1 = r1 - u1 * tt, q2 = r2 - u2 * tt;
                    const float radius = sqrtf(q0 * q0 + q1 * q1 + q2 * q2 + t[6] * t[6]);
                    const float uw = w == 0 ? u0 : w == 1 ? u1 : u2;
                    a += uw * (1e-7f * cz * (ash(tt / radius) - ash((tt - len) / radius)));
                } else if (kind < 1.5f) {
                    const float bw = w == 0 ? t[3] : w == 1 ? t[4] : t[5];
                    a += bw * (1e-7f * cz * (1.0f / sqrtf(r0 * r0 + r1 * r1 + r2 * r2 + t[6] * t[6])));
                } else {
                    const float b0 = t[3], b1 = t[4], b2 = t[5];
                    const float cw = w == 0 ? b1 * p[2] - b2 * p[1] : w == 1 ? b2 * p[0] - b0 * p[2]
                                                                      : b0 * p[1] - b1 * p[0];
                    a += 0.5f * cz * cw;
                }
            }
            acc = bi == 0 ? a : acc + a;
        }
    }
    if (i < D.E) out[i] = acc;
}

// Interleaves the planar work vectors into the reference's vec4 record
// (x, r, p, w) for inspection.
__global__ void k_em_pack_work(EmDev D, float4* out) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i < D.E) out[i] = make_float4(D.x[i], D.r[i], D.p[i], D.w[i]);
}

// motion (src/em/motion.wgsl:8-26): the conductivity-weighted u x B of the
// (up to) four cells around each edge, projected on the edge; fluid cells
// are FluidCell records (velocity at floats 0-2, mobile where float 12 >
// 0.5), B is this context's last cell result.
__global__ void __launch_bounds__(kBlock) k_em_motion(EmDev D, const float* __restrict__ fluid) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= D.E) return;
    int p[3], w;
    edge_decode(D, i, p, &w);
    const int a = (w + 1) % 3, b = (w + 2) % 3;
    const uint32_t d[3] = {D.n[0], D.n[1], D.n[2]};
    float weighted = 0.0f, sigma = 0.0f;
    for (int u = 0; u < 2; u++)
        for (int v = 0; v < 2; v++) {
            int q[3] = {p[0], p[1], p[2]};
            q[a] -= u;
            q[b] -= v;
            if (valid3(q, d)) {
                const uint32_t c = (uint32_t)q[0] + D.n[0] * ((uint32_t)q[1] + D.n[1] * (uint32_t)q[2]);
                const float sc = D.sig_c[c];
                sigma += sc;
                const float* f = fluid + (size_t)c * 16;
                if (f[12] > 0.5f) {
                    const float4 B = D.results[4 * (size_t)c];
                    const float cr = w == 0 ? f[1] * B.z - f[2] * B.y : w == 1 ? f[2] * B.x - f[0] * B.z
                                                                                 : f[0] * B.y - f[1] * B.x;
                    weighted += sc * cr;
                }
            }
        }
    D.emf[i] = weighted / fmx(sigma, 1e-30f);
}

__global__ void k_em_pack_coefficients(EmDev D, float4* out) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i < D.E) out[i] = make_float4(D.sig[i], D.diag[i], (float)D.flags[i], D.emf[i]);
}

}  // namespace

// ------------------------------------------------------------------ host
struct mhdproj_em_ctx {
    EmDev D{};
    mhdproj_em_config cfg{};
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaEvent_t ev = nullptr, t0 = nullptr, t1 = nullptr;
    std::vector<void*> allocs;
    float4* h_sc = nullptr;  // pinned copy of the scalars
    uint32_t* h_err = nullptr;
    float4* checkpoint = nullptr;
    float* d_props = nullptr;
    uint32_t props_cap = 0;
    float* d_elements = nullptr;
    uint32_t elements_cap = 0;
    float4* d_energy = nullptr;  // energy partials and result
    float4* d_body = nullptr;  // body partials and totals
    uint32_t body_cap = 0;
    float* h_body = nullptr;   // pinned totals
    cudaGraphExec_t batch = nullptr;  // kBatch CG iterations
    uint32_t batch_initial = 0;       // the step constants the batch graph was captured with
    uint32_t batch_nodal = 0;
    float batch_dt = 0.0f;
    bool materials = false;
    double time_s = 0.0, last_dt = 0.0;
    bool can_predict = false;
    float range[2] = {0.0f, 0.0f};
    uint64_t launches = 0;
    std::string err;
};

static std::string g_em_create_error;

static int em_fail(mhdproj_em_ctx* c, int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    else g_em_create_error = buf;
    return code;
}
#define EK(call)                                                                                    \
    do {                                                                                            \
        cudaError_t _e = (call);                                                                    \
        if (_e != cudaSuccess)                                                                      \
            return em_fail(ctx, _e == cudaErrorMemoryAllocation ? MHDPROJ_ERR_OUT_OF_MEMORY : MHDPROJ_ERR_CUDA, \
                           "%s: %s", #call, cudaGetErrorString(_e));                                \
    } while (0)

template <class T>
static cudaError_t em_alloc(mhdproj_em_ctx* ctx, T** p, size_t bytes) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, bytes ? bytes : 16);
    if (e != cudaSuccess) return e;
    ctx->allocs.push_back(q);
    *p = (T*)q;
    return cudaMemsetAsync(q, 0, bytes ? bytes : 16, ctx->stream);
}

static int em_wait(mhdproj_em_ctx* ctx, double timeout_s = 600.0) {
    EK(cudaEventRecord(ctx->ev, ctx->stream));
    auto t0 = std::chrono::steady_clock::now();
    int spins = 0;
    for (;;) {
        cudaError_t e = cudaEventQuery(ctx->ev);
        if (e == cudaSuccess) return 0;
        if (e != cudaErrorNotReady) return em_fail(ctx, MHDPROJ_ERR_CUDA, "stream wait: %s", cudaGetErrorString(e));
        if (++spins > 2000) std::this_thread::sleep_for(std::chrono::microseconds(50));
        else std::this_thread::yield();
        double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (el > timeout_s)
            return em_fail(ctx, MHDPROJ_ERR_TIMEOUT, "device work did not finish within %.0f s", timeout_s);
    }
}

static unsigned em_groups(uint32_t n) { return (n + kBlock - 1) / kBlock; }

#define EM_LAUNCH(kernel, n, ...)                                                  \
    do {                                                                           \
        kernel<<<em_groups(n) ? em_groups(n) : 1, kBlock, 0, ctx->stream>>>(__VA_ARGS__); \
        ctx->launches++;                                                           \
    } while (0)
#define EM_SINGLE(kernel, ...)                                   \
    do {                                                         \
        kernel<<<1, kBlock, 0, ctx->stream>>>(__VA_ARGS__);      \
        ctx->launches++;                                         \
    } while (0)

static int em_read_status(mhdproj_em_ctx* ctx) {
    EK(cudaMemcpyAsync(ctx->h_sc, ctx->D.scalars, 8 * sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream));
    return em_wait(ctx);
}
static bool status_finite(const float4* sc) {
    const float* v = &sc[0].x;
    for (int k = 0; k < 8; k++)
        if (!std::isfinite(v[k])) return false;
    return true;
}
static uint32_t em_nodes(const EmDev& D) { return (D.n[0] + 1) * (D.n[1] + 1) * (D.n[2] + 1); }
// append_nodal (src/em/mod.rs:639-659)
static void em_append_nodal(mhdproj_em_ctx* ctx, bool initial) {
    const EmDev& D = ctx->D;
    if (!D.nodal) return;
    if (initial) {
        EM_LAUNCH(k_em_nodal_build<true>, em_nodes(D), D, em_nodes(D));
        EM_LAUNCH(k_em_nodal<true>, D.E, D);
    } else {
        EM_LAUNCH(k_em_nodal_build<false>, em_nodes(D), D, em_nodes(D));
        EM_LAUNCH(k_em_nodal<false>, D.E, D);
    }
}
static void em_iteration(mhdproj_em_ctx* ctx) {
    const EmDev& D = ctx->D;
    EM_LAUNCH(k_em_apply<true>, D.E, D);
    EM_SINGLE(k_em_alpha_reduce, D);
    EM_LAUNCH(k_em_update_residual, D.E, D);
    em_append_nodal(ctx, false);
    EM_SINGLE(k_em_beta_reduce, D);
    EM_LAUNCH(k_em_update_search, D.E, D);
}
// The iteration kernels take EmDev by value, so the graph holds the step
// constants they read (initial, dt, nodal mode); it is captured again when
// they change.
static int em_build_batch(mhdproj_em_ctx* ctx) {
    if (ctx->batch && ctx->batch_initial == ctx->D.initial && ctx->batch_dt == ctx->D.dt &&
        ctx->batch_nodal == ctx->D.nodal)
        return 0;
    if (ctx->batch) {
        cudaGraphExecDestroy(ctx->batch);
        ctx->batch = nullptr;
    }
    if (!ctx->stream) return 0;  // the legacy default stream cannot be captured: launch directly
    cudaGraph_t g = nullptr;
    EK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const uint64_t before = ctx->launches;
    for (uint32_t k = 0; k < kBatch; k++) em_iteration(ctx);
    ctx->launches = before;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (e != cudaSuccess) return em_fail(ctx, MHDPROJ_ERR_CUDA, "batch capture: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&ctx->batch, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return em_fail(ctx, MHDPROJ_ERR_CUDA, "batch instantiate: %s", cudaGetErrorString(e));
    ctx->batch_initial = ctx->D.initial;
    ctx->batch_nodal = ctx->D.nodal;
    ctx->batch_dt = ctx->D.dt;
    return 0;
}
static void em_prepare(mhdproj_em_ctx* ctx) {
    EM_LAUNCH(k_em_prepare, ctx->D.E, ctx->D);
    em_append_nodal(ctx, true);
    EM_SINGLE(k_em_initial_reduce, ctx->D);
}
static void em_restart(mhdproj_em_ctx* ctx) {
    EM_LAUNCH(k_em_true_residual, ctx->D.E, ctx->D);
    em_append_nodal(ctx, true);
    EM_SINGLE(k_em_restart_reduce, ctx->D);
}

extern "C" {

const char* mhdproj_em_last_error(const mhdproj_em_ctx* ctx) {
    return ctx ? ctx->err.c_str() : g_em_create_error.c_str();
}

void mhdproj_em_destroy(mhdproj_em_ctx* ctx) {
    if (!ctx) return;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->batch) cudaGraphExecDestroy(ctx->batch);
    for (void* p : ctx->allocs) cudaFree(p);
    if (ctx->h_sc) cudaFreeHost(ctx->h_sc);
    if (ctx->h_err) cudaFreeHost(ctx->h_err);
    if (ctx->h_body) cudaFreeHost(ctx->h_body);
    if (ctx->ev) cudaEventDestroy(ctx->ev);
    if (ctx->t0) cudaEventDestroy(ctx->t0);
    if (ctx->t1) cudaEventDestroy(ctx->t1);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

int mhdproj_em_create(const mhdproj_em_config* cfg, mhdproj_em_ctx** out) {
    mhdproj_em_ctx* ctx = nullptr;
    if (!cfg || !out) return em_fail(nullptr, MHDPROJ_ERR_INVALID, "null argument");
    *out = nullptr;
    if (cfg->nx == 0 || cfg->ny == 0 || cfg->nz == 0)
        return em_fail(nullptr, MHDPROJ_ERR_INVALID, "EM grid dimensions must be positive");
    if (!(cfg->cell_m > 0.0f) || !std::isfinite(cfg->cell_m))
        return em_fail(nullptr, MHDPROJ_ERR_INVALID, "EM cell size must be positive and finite");
    if (!(cfg->dt_s > 0.0) || !std::isfinite(cfg->dt_s))
        return em_fail(nullptr, MHDPROJ_ERR_INVALID, "EM time step must be positive and finite");
    if (!(cfg->relative_tolerance > 0.0f) || cfg->max_iterations == 0)
        return em_fail(nullptr, MHDPROJ_ERR_INVALID, "EM tolerance and iteration cap must be positive");
    if (cfg->mode != MHDPROJ_EM_INDUCTION && cfg->mode != MHDPROJ_EM_APPLIED)
        return em_fail(nullptr, MHDPROJ_ERR_INVALID, "unknown EM mode %d", cfg->mode);
    const uint64_t x = cfg->nx, y = cfg->ny, z = cfg->nz;
    const uint64_t counts[3] = {x * (y + 1) * (z + 1), (x + 1) * y * (z + 1), (x + 1) * (y + 1) * z};
    const uint64_t total = counts[0] + counts[1] + counts[2];
    if (total > 0xFFFFFFFFull || x * y * z > 0xFFFFFFFFull)  // grid.rs:25-27
        return em_fail(nullptr, MHDPROJ_ERR_INVALID, "EM grid indexing exceeds u32");
    ctx = new mhdproj_em_ctx();
    ctx->cfg = *cfg;
    EmDev& D = ctx->D;
    D.n[0] = cfg->nx;
    D.n[1] = cfg->ny;
    D.n[2] = cfg->nz;
    D.cells = (uint32_t)(x * y * z);
    for (int k = 0; k < 3; k++) D.e[k] = (uint32_t)counts[k];
    D.E = (uint32_t)total;
    D.initial = 1;
    D.pf = 0.0f;
    D.dt = 1e-5f;  // grid.rs:34; advance sets the configured step
    D.mu0 = 4e-7f * 3.14159265358979323846f;
    D.h = cfg->cell_m;
    D.tol2 = 1e-10f;
    D.vacuum = cfg->mode == MHDPROJ_EM_APPLIED ? 1u : 0u;
    for (int k = 0; k < 3; k++) D.origin[k] = cfg->origin_m[k];
    auto bail = [&](int code) {
        mhdproj_em_destroy(ctx);
        return code;
    };
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        em_fail(nullptr, MHDPROJ_ERR_CUDA, "stream: %s", cudaGetErrorString(e));
        delete ctx;
        return MHDPROJ_ERR_CUDA;
    }
    ctx->own_stream = true;
    const size_t E = D.E, C = D.cells;
    const size_t groups = std::max(em_groups(D.E), em_groups(D.cells));
    cudaError_t es[40];
    int ne = 0;
    es[ne++] = cudaEventCreateWithFlags(&ctx->ev, cudaEventDisableTiming);
    es[ne++] = cudaEventCreate(&ctx->t0);
    es[ne++] = cudaEventCreate(&ctx->t1);
    es[ne++] = em_alloc(ctx, &D.as, E * 4);
    es[ne++] = em_alloc(ctx, &D.asp, E * 4);
    es[ne++] = em_alloc(ctx, &D.sig, E * 4);
    es[ne++] = em_alloc(ctx, &D.diag, E * 4);
    es[ne++] = em_alloc(ctx, &D.emf, E * 4);
    es[ne++] = em_alloc(ctx, &D.flags, E);
    es[ne++] = em_alloc(ctx, &D.x, E * 4);
    es[ne++] = em_alloc(ctx, &D.r, E * 4);
    es[ne++] = em_alloc(ctx, &D.p, E * 4);
    es[ne++] = em_alloc(ctx, &D.w, E * 4);
    es[ne++] = em_alloc(ctx, &D.prev, E * 4);
    es[ne++] = em_alloc(ctx, &D.sig_c, C * 4);
    es[ne++] = em_alloc(ctx, &D.mu_c, C * 4);
    for (int a = 0; a < 3; a++) {
        uint64_t f = (x + (a == 0)) * (y + (a == 1)) * (z + (a == 2));
        es[ne++] = em_alloc(ctx, &D.nu[a], f * 4);
    }
    es[ne++] = em_alloc(ctx, &D.nv, (x + 1) * (y + 1) * (z + 1) * 4);
    es[ne++] = em_alloc(ctx, &D.partials, (4 * groups + 4) * sizeof(float4));
    es[ne++] = em_alloc(ctx, &D.scalars, 8 * sizeof(float4));
    es[ne++] = em_alloc(ctx, &D.results, 4 * C * sizeof(float4));
    es[ne++] = em_alloc(ctx, &ctx->checkpoint, 4 * C * sizeof(float4));
    es[ne++] = em_alloc(ctx, &D.err, 16);
    es[ne++] = cudaMallocHost(&ctx->h_sc, 8 * sizeof(float4));
    es[ne++] = cudaMallocHost(&ctx->h_err, 16);
    for (int k = 0; k < ne; k++)
        if (es[k] != cudaSuccess) {
            em_fail(nullptr, es[k] == cudaErrorMemoryAllocation ? MHDPROJ_ERR_OUT_OF_MEMORY : MHDPROJ_ERR_CUDA,
                    "EM workspace (%.0f MiB): %s", (double)(E * 45 + C * 136) / 1048576.0,
                    cudaGetErrorString(es[k]));
            return bail(es[k] == cudaErrorMemoryAllocation ? MHDPROJ_ERR_OUT_OF_MEMORY : MHDPROJ_ERR_CUDA);
        }
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        em_fail(nullptr, MHDPROJ_ERR_CUDA, "EM workspace: %s", cudaGetErrorString(e));
        return bail(MHDPROJ_ERR_CUDA);
    }
    *out = ctx;
    return 0;
}

// The EmConfig fields a caller may change between steps (dt_s,
// relative_tolerance, max_iterations) and the nodal switch point; the grid,
// origin and mode are fixed at creation.
int mhdproj_em_update_config(mhdproj_em_ctx* ctx, const mhdproj_em_config* cfg) {
    if (!ctx || !cfg) return MHDPROJ_ERR_INVALID;
    if (!(cfg->dt_s > 0.0) || !std::isfinite(cfg->dt_s))
        return em_fail(ctx, MHDPROJ_ERR_INVALID, "EM time step must be positive and finite");
    if (!(cfg->relative_tolerance > 0.0f) || cfg->max_iterations == 0)
        return em_fail(ctx, MHDPROJ_ERR_INVALID, "EM tolerance and iteration cap must be positive");
    ctx->cfg.dt_s = cfg->dt_s;
    ctx->cfg.relative_tolerance = cfg->relative_tolerance;
    ctx->cfg.max_iterations = cfg->max_iterations;
    ctx->cfg.nodal_switch_after = cfg->nodal_switch_after;
    return 0;
}

int mhdproj_em_set_stream(mhdproj_em_ctx* ctx, void* stream) {
    if (!ctx) return MHDPROJ_ERR_INVALID;
    EK(cudaStreamSynchronize(ctx->stream));
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    ctx->own_stream = false;
    ctx->stream = (cudaStream_t)stream;
    return 0;
}

int mhdproj_em_sizes(const mhdproj_em_ctx* ctx, uint64_t out[8]) {
    if (!ctx || !out) return MHDPROJ_ERR_INVALID;
    const EmDev& D = ctx->D;
    out[0] = D.n[0];
    out[1] = D.n[1];
    out[2] = D.n[2];
    out[3] = D.cells;
    out[4] = D.e[0];
    out[5] = D.e[1];
    out[6] = D.e[2];
    out[7] = D.E;
    return 0;
}

int mhdproj_em_set_materials(mhdproj_em_ctx* ctx, const uint32_t* materials, const float* properties,
                             uint32_t count, float conductivity_range[2]) {
    if (!ctx) return MHDPROJ_ERR_INVALID;
    if (!materials || !properties || count == 0)
        return em_fail(ctx, MHDPROJ_ERR_INVALID, "materials and at least one property row are required");
    for (uint32_t k = 0; k < 2 * count; k++)
        if (!std::isfinite(properties[k]))
            return em_fail(ctx, MHDPROJ_ERR_INVALID, "material properties must be finite");
    EmDev& D = ctx->D;
    if (count > ctx->props_cap) {
        float* p = nullptr;
        EK(em_alloc(ctx, &p, (size_t)count * 8));
        ctx->d_props = p;
        ctx->props_cap = count;
    }
    EK(cudaMemcpyAsync(ctx->d_props, properties, (size_t)count * 8, cudaMemcpyHostToDevice, ctx->stream));
    D.materials = materials;
    D.props = ctx->d_props;
    D.n_props = count;
    EK(cudaMemsetAsync(D.err, 0, 4, ctx->stream));
    EM_LAUNCH(k_em_cells, D.cells, D);
    for (int a = 0; a < 3; a++) {
        const uint32_t f = (D.n[0] + (a == 0)) * (D.n[1] + (a == 1)) * (D.n[2] + (a == 2));
        EM_LAUNCH(k_em_faces, f, D, a, f);
    }
    EM_LAUNCH(k_em_coefficients, D.E, D);
    EM_SINGLE(k_em_coefficient_check, D);
    EK(cudaGetLastError());
    EK(cudaMemcpyAsync(ctx->h_sc, D.scalars, sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream));
    EK(cudaMemcpyAsync(ctx->h_err, D.err, 4, cudaMemcpyDeviceToHost, ctx->stream));
    int rc = em_wait(ctx);
    if (rc) return rc;
    D.materials = nullptr;
    const float4 check = ctx->h_sc[0];
    ctx->range[0] = check.w > 0.0f ? check.y : 0.0f;
    ctx->range[1] = check.z;
    if (conductivity_range) {
        conductivity_range[0] = ctx->range[0];
        conductivity_range[1] = ctx->range[1];
    }
    if (*ctx->h_err) return em_fail(ctx, MHDPROJ_ERR_INVALID, "a material id has no property row");
    ctx->materials = true;
    if (check.x > 0.0f)  // mod.rs:563-567 and :748-752
        return em_fail(ctx, MHDPROJ_ERR_INVALID,
                       "A conductor touches the EM outer boundary; add air padding to the domain");
    return 0;
}

int mhdproj_em_set_motional_emf(mhdproj_em_ctx* ctx, const float* emf) {
    if (!ctx) return MHDPROJ_ERR_INVALID;
    if (emf) EK(cudaMemcpyAsync(ctx->D.emf, emf, (size_t)ctx->D.E * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    else EK(cudaMemsetAsync(ctx->D.emf, 0, (size_t)ctx->D.E * 4, ctx->stream));
    return em_wait(ctx);
}

// EmState::energy_step (src/em/mod.rs:1106-1133): the energy ledger of the
// last committed step.
int mhdproj_em_energy(mhdproj_em_ctx* ctx, double out[7]) {
    if (!ctx || !out) return MHDPROJ_ERR_INVALID;
    if (!ctx->materials) return em_fail(ctx, MHDPROJ_ERR_STATE, "set the EM materials first");
    const EmDev& D = ctx->D;
    const uint32_t ng = em_groups(D.E);
    if (!ctx->d_energy) {
        float4* p = nullptr;
        EK(em_alloc(ctx, &p, (2 * (size_t)ng + 2) * sizeof(float4)));
        ctx->d_energy = p;
    }
    float4* res = ctx->d_energy + 2 * (size_t)ng;
    k_em_energy_collect<<<ng, kBlock, 0, ctx->stream>>>(D, ctx->d_energy);
    k_em_energy_reduce<<<1, kBlock, 0, ctx->stream>>>(D, ctx->d_energy, res);
    ctx->launches += 2;
    EK(cudaGetLastError());
    EK(cudaMemcpyAsync(ctx->h_sc + 6, res, 2 * sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream));
    int rc = em_wait(ctx);
    if (rc) return rc;
    const float* v = &ctx->h_sc[6].x;
    for (int k = 0; k < 8; k++)
        if (!std::isfinite(v[k])) return em_fail(ctx, MHDPROJ_ERR_NONFINITE, "Nonfinite EM energy integral");
    for (int k = 0; k < 6; k++) out[k] = v[k];
    out[6] = 0.0;
    if (ctx->time_s == 0.0) {
        for (int k = 1; k < 7; k++) out[k] = 0.0;
        return 0;
    }
    out[6] = out[5] - out[1] - out[2] - out[3] - out[4];
    return 0;
}

// Per-body force and power of the last accepted step (body-stats.wgsl).
int mhdproj_em_body_forces(mhdproj_em_ctx* ctx, const uint32_t* masks, uint32_t bodies, float* totals) {
    if (!ctx || !masks || !totals || bodies == 0 || bodies > 32)
        return em_fail(ctx, MHDPROJ_ERR_INVALID, "body masks hold 1..32 bodies");
    const EmDev& D = ctx->D;
    const uint32_t ng = em_groups(D.cells);
    if (bodies > ctx->body_cap) {
        float4* p = nullptr;
        EK(em_alloc(ctx, &p, ((size_t)bodies * ng + bodies) * sizeof(float4)));
        ctx->d_body = p;
        if (ctx->h_body) cudaFreeHost(ctx->h_body);
        ctx->h_body = nullptr;
        EK(cudaMallocHost(&ctx->h_body, (size_t)bodies * 16));
        ctx->body_cap = bodies;
    }
    float4* totals_d = ctx->d_body + (size_t)bodies * ng;
    k_em_body_collect<<<dim3(ng, 1, bodies), kBlock, 0, ctx->stream>>>(D, masks, ctx->d_body);
    k_em_body_reduce<<<dim3(1, 1, bodies), kBlock, 0, ctx->stream>>>(D, ctx->d_body, totals_d);
    ctx->launches += 2;
    EK(cudaGetLastError());
    EK(cudaMemcpyAsync(ctx->h_body, totals_d, (size_t)bodies * 16, cudaMemcpyDeviceToHost, ctx->stream));
    int rc = em_wait(ctx);
    if (rc) return rc;
    memcpy(totals, ctx->h_body, (size_t)bodies * 16);
    return 0;
}

// The source pass over host-side elements (12 floats each), into `applied`
// (device, one float per edge).
int mhdproj_em_evaluate_sources(mhdproj_em_ctx* ctx, const float* elements, uint32_t count, float* applied) {
    if (!ctx || !applied || (count && !elements)) return MHDPROJ_ERR_INVALID;
    if (count > 1000000u)  // src/em/sources.rs:330-336
        return em_fail(ctx, MHDPROJ_ERR_INVALID, "Source discretization is too large or has nonfinite values");
    for (size_t k = 0; k < 12 * (size_t)count; k++)
        if (!std::isfinite(elements[k]))
            return em_fail(ctx, MHDPROJ_ERR_INVALID, "Source discretization is too large or has nonfinite values");
    if ((uint64_t)ctx->D.E * count > 50000000000ull)  // src/em/mod.rs:208-210
        return em_fail(ctx, MHDPROJ_ERR_INVALID,
                       "Direct source summation exceeds the work budget for this grid; reduce source refinement/"
                       "segment count or increase cell spacing");
    if (count > ctx->elements_cap) {
        float* p = nullptr;
        EK(em_alloc(ctx, &p, (size_t)count * 48));
        ctx->d_elements = p;
        ctx->elements_cap = count;
    }
    if (count) EK(cudaMemcpyAsync(ctx->d_elements, elements, (size_t)count * 48, cudaMemcpyHostToDevice, ctx->stream));
    EM_LAUNCH(k_em_source_eval, ctx->D.E, ctx->D, ctx->d_elements, count, applied);
    EK(cudaGetLastError());
    return em_wait(ctx);
}

// EmState::set_velocity (src/em/mod.rs:757-834): the lagged motional EMF
// from the fluid's cell records and the B of the last accepted step.
int mhdproj_em_set_motion(mhdproj_em_ctx* ctx, const float* fluid_cells) {
    if (!ctx || !fluid_cells) return MHDPROJ_ERR_INVALID;
    if (!ctx->materials) return em_fail(ctx, MHDPROJ_ERR_STATE, "set the EM materials first");
    EM_LAUNCH(k_em_motion, ctx->D.E, ctx->D, fluid_cells);
    EK(cudaGetLastError());
    return em_wait(ctx);
}

int mhdproj_em_set_reaction(mhdproj_em_ctx* ctx, const float* a) {
    if (!ctx || !a) return MHDPROJ_ERR_INVALID;
    EK(cudaMemcpyAsync(ctx->D.x, a, (size_t)ctx->D.E * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    return em_wait(ctx);
}

int mhdproj_em_copy(mhdproj_em_ctx* ctx, int which, float* out) {
    if (!ctx || !out) return MHDPROJ_ERR_INVALID;
    const EmDev& D = ctx->D;
    const size_t E = D.E, C = D.cells;
    switch (which) {
        case MHDPROJ_EM_REACTION:
            EK(cudaMemcpyAsync(out, D.x, E * 4, cudaMemcpyDeviceToDevice, ctx->stream));
            break;
        case MHDPROJ_EM_PREVIOUS:
            EK(cudaMemcpyAsync(out, D.prev, E * 4, cudaMemcpyDeviceToDevice, ctx->stream));
            break;
        case MHDPROJ_EM_APPLIED_POTENTIAL:
            EK(cudaMemcpyAsync(out, D.as, E * 4, cudaMemcpyDeviceToDevice, ctx->stream));
            break;
        case MHDPROJ_EM_CELLS:
            EK(cudaMemcpyAsync(out, D.results, C * 64, cudaMemcpyDeviceToDevice, ctx->stream));
            break;
        case MHDPROJ_EM_WORK:
            EM_LAUNCH(k_em_pack_work, D.E, D, (float4*)out);
            break;
        case MHDPROJ_EM_EDGE_COEFFICIENTS:
            EM_LAUNCH(k_em_pack_coefficients, D.E, D, (float4*)out);
            break;
        default:
            return em_fail(ctx, MHDPROJ_ERR_INVALID, "unknown EM array %d", which);
    }
    EK(cudaGetLastError());
    return em_wait(ctx);
}

int mhdproj_em_apply_operator(mhdproj_em_ctx* ctx, const float* p, float* q, int air_stencil) {
    if (!ctx || !p || !q) return MHDPROJ_ERR_INVALID;
    if (!ctx->materials) return em_fail(ctx, MHDPROJ_ERR_STATE, "set the EM materials first");
    EmDev& D = ctx->D;
    EK(cudaMemcpyAsync(D.p, p, (size_t)D.E * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    EK(cudaMemsetAsync(D.scalars, 0, 8 * sizeof(float4), ctx->stream));
    if (air_stencil) EM_LAUNCH(k_em_apply<true>, D.E, D);
    else EM_LAUNCH(k_em_apply<false>, D.E, D);
    EK(cudaGetLastError());
    EK(cudaMemcpyAsync(q, D.w, (size_t)D.E * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    return em_wait(ctx);
}

// EmState::advance_to (src/em/mod.rs:863-1090) without the source summation:
// `applied` is A_s at time_s (device, one float per edge) or NULL when the
// applied field is unchanged.
int mhdproj_em_advance(mhdproj_em_ctx* ctx, double time_s, int initial, const float* applied,
                       mhdproj_em_diagnostics* diag) {
    if (!ctx) return MHDPROJ_ERR_INVALID;
    if (!ctx->materials) return em_fail(ctx, MHDPROJ_ERR_STATE, "set the EM materials first");
    if (!std::isfinite(time_s)) return em_fail(ctx, MHDPROJ_ERR_INVALID, "EM time must be finite");
    if (ctx->cfg.mode == MHDPROJ_EM_APPLIED && (!initial || time_s < 0.0))  // mod.rs:841-858
        return em_fail(ctx, MHDPROJ_ERR_INVALID, "Applied field time must be nonnegative and mode Applied");
    const auto started = std::chrono::steady_clock::now();
    EmDev& D = ctx->D;
    D.initial = initial ? 1u : 0u;
    float pf = 0.0f;
    if (!initial && ctx->can_predict && ctx->last_dt > 0.0) {
        const float ratio = (float)((time_s - ctx->time_s) / ctx->last_dt);
        pf = (std::isfinite(ratio) && ratio > 0.0f) ? ratio : 0.0f;
    }
    D.pf = pf;
    D.dt = (float)ctx->cfg.dt_s;
    D.tol2 = ctx->cfg.relative_tolerance * ctx->cfg.relative_tolerance;
    const uint32_t switch_after = ctx->cfg.nodal_switch_after;
    const bool allow_nodal = !initial && ctx->cfg.mode == MHDPROJ_EM_INDUCTION && ctx->cfg.max_iterations > switch_after;
    // each step starts in Jacobi mode; a zero switch point starts in nodal
    // mode (src/em/mod.rs:897-903)
    D.nodal = (allow_nodal && switch_after == 0) ? 1u : 0u;
    EK(cudaEventRecord(ctx->t0, ctx->stream));
    EM_LAUNCH(k_em_sources, D.E, D, applied);
    EM_LAUNCH(k_em_begin_step, D.E, D);
    em_prepare(ctx);
    EK(cudaGetLastError());
    int rc = em_read_status(ctx);
    if (rc) return rc;
    if (ctx->h_sc[1].x != 0.0f) {  // initial_reduce chose a power-of-two normalisation
        em_prepare(ctx);
        if ((rc = em_read_status(ctx))) return rc;
    }
    if (pf > 0.0f && (!status_finite(ctx->h_sc) || ctx->h_sc[0].y > ctx->h_sc[0].z)) {
        D.pf = 0.0f;
        EM_LAUNCH(k_em_zero_guess, D.E, D);
        em_prepare(ctx);
        if ((rc = em_read_status(ctx))) return rc;
    }
    rc = em_build_batch(ctx);
    if (rc) return rc;
    auto its = [&]() { return (uint32_t)ctx->h_sc[1].z; };
    const uint32_t cap = ctx->cfg.max_iterations;
    for (;;) {
        while (ctx->h_sc[1].w == 0.0f && status_finite(ctx->h_sc) && its() < cap) {
            const uint32_t batch = std::min(cap - its(), kBatch);
            if (batch == kBatch && ctx->batch) {
                EK(cudaGraphLaunch(ctx->batch, ctx->stream));
                ctx->launches += 5 * kBatch;
            } else {
                for (uint32_t k = 0; k < batch; k++) em_iteration(ctx);
            }
            EK(cudaGetLastError());
            if ((rc = em_read_status(ctx))) return rc;
            // switch to the nodal correction at a true-residual restart
            // (src/em/mod.rs:966-990); the batch graph is captured again
            if (allow_nodal && !D.nodal && ctx->h_sc[1].w == 0.0f && status_finite(ctx->h_sc) &&
                its() >= switch_after && its() < cap) {
                D.nodal = 1;
                em_restart(ctx);
                if ((rc = em_read_status(ctx))) return rc;
                if ((rc = em_build_batch(ctx))) return rc;
            }
        }
        if (ctx->h_sc[1].w != 1.0f) break;
        em_restart(ctx);
        if ((rc = em_read_status(ctx))) return rc;
        if (ctx->h_sc[1].w == 1.0f || its() >= cap) break;
    }
    if (ctx->h_sc[1].w != 1.0f && status_finite(ctx->h_sc)) {
        em_restart(ctx);
        if ((rc = em_read_status(ctx))) return rc;
    }
    float status[8];
    memcpy(status, ctx->h_sc, sizeof status);
    if (diag) {
        memset(diag, 0, sizeof *diag);
        memcpy(diag->status, status, sizeof status);
        diag->iterations = (uint32_t)status[6];
        diag->relative_residual = std::sqrt(status[1] / std::max(status[2], 1e-38f));
        diag->conductivity_range[0] = ctx->range[0];
        diag->conductivity_range[1] = ctx->range[1];
    }
    if (status[7] != 1.0f || !status_finite(ctx->h_sc)) {
        EM_LAUNCH(k_em_rollback, D.E, D);
        ctx->can_predict = false;
        rc = em_wait(ctx);
        if (rc) return rc;
        return em_fail(ctx, MHDPROJ_ERR_NOT_CONVERGED,
                       "EM solve did not converge: %u iterations, true relative residual %.3e (requested %.3e); "
                       "conducting-edge sigma range %.3e..%.3e S/m; state restored",
                       (uint32_t)status[6], std::sqrt(status[1] / std::max(status[2], 1e-38f)),
                       ctx->cfg.relative_tolerance, ctx->range[0], ctx->range[1]);
    }
    EK(cudaMemcpyAsync(ctx->checkpoint, D.results, (size_t)D.cells * 64, cudaMemcpyDeviceToDevice, ctx->stream));
    EM_LAUNCH(k_em_fields, D.cells, D);
    EM_SINGLE(k_em_field_reduce, D);
    EM_LAUNCH(k_em_commit, D.E, D);
    EK(cudaEventRecord(ctx->t1, ctx->stream));
    EK(cudaGetLastError());
    if ((rc = em_read_status(ctx))) return rc;
    const float* stats = &ctx->h_sc[2].x;
    bool finite = true;
    for (int k = 0; k < 16; k++) finite = finite && std::isfinite(stats[k]);
    if (!finite) {
        EM_LAUNCH(k_em_rollback, D.E, D);
        EK(cudaMemcpyAsync(D.results, ctx->checkpoint, (size_t)D.cells * 64, cudaMemcpyDeviceToDevice,
                           ctx->stream));
        ctx->can_predict = false;
        rc = em_wait(ctx);
        if (rc) return rc;
        return em_fail(ctx, MHDPROJ_ERR_NONFINITE, "Nonfinite EM field output; state restored");
    }
    ctx->last_dt = initial ? 0.0 : time_s - ctx->time_s;
    ctx->can_predict = !initial && status[2] > 0.0f;
    ctx->time_s = time_s;
    if (diag) {
        memcpy(diag->maxima, stats, 16);
        memcpy(diag->force_n, stats + 4, 12);
        diag->power_w = stats[7];
        diag->divergence_j_scaled = stats[8];
        diag->max_edge_j = stats[9];
        diag->divergence_b_scaled = stats[10];
        diag->magnetic_energy_j = stats[11];
        diag->applied_max_t = stats[12];
        diag->reaction_max_t = stats[13];
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, ctx->t0, ctx->t1);
        diag->device_ms = ms;
        diag->elapsed_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - started).count();
    }
    return 0;
}

int mhdproj_em_kernel_launches(const mhdproj_em_ctx* ctx, uint64_t* count) {
    if (!ctx || !count) return MHDPROJ_ERR_INVALID;
    *count = ctx->launches;
    return 0;
}

}  // extern "C"
