// reference_kernels.cu -- the reference solver on the GPU.
//
// The reference's own projection algorithm, for drop-in parity: FP32
// Jacobi-CG below 96^3 cells and aggregation-multigrid CG at or above
// (src/fluid/mod.rs:1015-1115, src/fluid/multigrid.rs), pinned gauge cells or
// mean-free residuals (configure_pressure_projection, :978-1002;
// pressure_subspace.wgsl), the reference's convergence tests, batching and
// 64-iteration physical check, warm start (pressure_warm/pressure_commit).
// Every kernel restates one WGSL entry point of src/fluid/solver.wgsl,
// multigrid.wgsl or pressure_subspace.wgsl; the comments name it.
//
// Arithmetic follows the reference's operation order with no fused
// multiply-add (this unit is compiled with -fmad=false), and reductions replay
// the reference's 256-lane workgroup tree and 256-stride final pass, so the
// results match the CPU restatement in oracle/ bit for bit.  Candidate
// velocities are the SoA face arrays of include/mhdproj.h; the coefficient
// cache and the PCG state keep the reference's vec4 lanes (cache: beta_x,
// beta_y, beta_z of the low faces, diagonal; work: x potential, y residual,
// z search, w product / diagonal / correction).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "reference.h"
#include "topology.h"

namespace mhdproj {

namespace {

constexpr int WG = 256;           // the reference's workgroup size
constexpr uint32_t COARSE_SWEEPS = 8;  // multigrid.rs:3
constexpr uint32_t MIN_CELLS = 96u * 96u * 96u;  // multigrid.rs:4

// Projection lanes of Params (src/fluid/mod.rs:120-130).
struct RParams {
    uint32_t dims[4], faces[4], flags[4];
    float physical[4], initial[4], solve[4], surface[4];
};

struct RView {
    RParams p;
    const uint32_t* mask;
    const float* occ;
    const float* phase;
    const float* oldp;
    const float* us[3];  // candidate velocities (SoA) as read by face(star)
    float4* cache;
    float4* work;
    float4* partials;
    float4* scalars;
};

struct I3 {
    int v[3];
};

__device__ __forceinline__ int32_t wrap_periodic(int32_t value, uint32_t size) {  // periodic.wgsl:5
    if (value >= 0) return (int32_t)((uint32_t)value % size);
    const uint32_t magnitude = (uint32_t)(-(value + 1)) + 1u;
    const uint32_t remainder = magnitude % size;
    return (int32_t)(remainder == 0u ? 0u : size - remainder);
}
__device__ __forceinline__ uint32_t idx3(I3 q, const uint32_t* d) {
    return (uint32_t)q.v[0] + d[0] * ((uint32_t)q.v[1] + d[1] * (uint32_t)q.v[2]);
}
__device__ __forceinline__ I3 decode3(uint32_t i, const uint32_t* d) {
    I3 q;
    q.v[0] = (int)(i % d[0]);
    q.v[1] = (int)((i / d[0]) % d[1]);
    q.v[2] = (int)(i / (d[0] * d[1]));
    return q;
}
__device__ __forceinline__ I3 wrap_cell(const RParams& p, I3 q) {
    for (int a = 0; a < 3; a++)
        if (p.flags[0] & (1u << a)) q.v[a] = wrap_periodic(q.v[a], p.dims[a]);
    return q;
}
__device__ __forceinline__ bool valid_cell(const RParams& p, I3 q) {
    for (int a = 0; a < 3; a++)
        if (q.v[a] < 0 || q.v[a] >= (int)p.dims[a]) return false;
    return true;
}
__device__ __forceinline__ bool fluid(const RView& s, I3 pos) {
    const I3 q = wrap_cell(s.p, pos);
    if (!valid_cell(s.p, q)) return false;
    return s.mask[idx3(q, s.p.dims)] != 0u;
}
__device__ __forceinline__ bool valid_face(const RParams& p, I3 q, int axis) {
    for (int a = 0; a < 3; a++) {
        const int lim = (int)p.dims[a] + (a == axis ? 1 : 0);
        if (q.v[a] < 0 || q.v[a] >= lim) return false;
    }
    return true;
}
__device__ __forceinline__ bool open_face(const RView& s, I3 pos, int axis) {  // solver.wgsl:32
    const I3 q = wrap_cell(s.p, pos);
    if (!valid_face(s.p, q, axis)) return false;
    I3 left = q;
    left.v[axis] -= 1;
    return fluid(s, left) && fluid(s, q);
}
// Index of face position q (canonical, valid) of the axis in its SoA array.
__device__ __forceinline__ uint32_t face_index(const RParams& p, I3 q, int axis) {
    const uint32_t nx = p.dims[0], ny = p.dims[1];
    if (axis == 0) return (uint32_t)q.v[0] + (nx + 1) * ((uint32_t)q.v[1] + ny * (uint32_t)q.v[2]);
    if (axis == 1) return (uint32_t)q.v[0] + nx * ((uint32_t)q.v[1] + (ny + 1) * (uint32_t)q.v[2]);
    return (uint32_t)q.v[0] + nx * ((uint32_t)q.v[1] + ny * (uint32_t)q.v[2]);
}
__device__ __forceinline__ float face_star(const RView& s, I3 pos, int axis) {  // face(pos, axis, true)
    const I3 q = wrap_cell(s.p, pos);
    if (!open_face(s, q, axis)) return 0.0f;
    return s.us[axis][face_index(s.p, q, axis)];
}
__device__ __forceinline__ float potential(const RView& s, I3 pos, int kind) {  // :37-39
    const I3 q = wrap_cell(s.p, pos);
    if (!valid_cell(s.p, q) || !fluid(s, q)) return 0.0f;
    const float4 v = s.work[idx3(q, s.p.dims)];
    return kind == 0 ? v.x : v.z;
}
__device__ __forceinline__ float occupancy(const RView& s, I3 pos) {
    const I3 q = wrap_cell(s.p, pos);
    if (!valid_cell(s.p, q)) return 0.0f;
    return s.occ[idx3(q, s.p.dims)];
}
__device__ __forceinline__ float density(const RView& s, I3 pos) {  // mix(e1,e2,t) = e1*(1-t)+e2*t
    const float t = occupancy(s, pos);
    return s.p.surface[1] * (1.0f - t) + s.p.physical[3] * t;
}
__device__ __forceinline__ float face_density(const RView& s, I3 pos, int axis) {
    I3 left = pos;
    left.v[axis] -= 1;
    return 0.5f * (density(s, left) + density(s, pos));
}
__device__ __forceinline__ float mobility(const RView& s, I3 pos, int axis) {  // :43-51
    const RParams& p = s.p;
    float beta = 1.0f;
    I3 left = pos;
    left.v[axis] -= 1;
    if (p.surface[0] > 0.5f) beta = p.physical[3] / face_density(s, pos, axis);
    if (p.flags[3] == 0u) return beta;
    if (!fluid(s, pos) || !fluid(s, left)) return 0.0f;
    const float fa = s.phase[idx3(wrap_cell(p, pos), p.dims)];
    const float fb = s.phase[idx3(wrap_cell(p, left), p.dims)];
    const float f = fminf(fa, fb);
    const float drag = p.solve[3] * (1.0f - f) * (1.0f - f) / (f * f * f + 1e-3f);
    return beta / (1.0f + p.physical[1] * drag);
}
__device__ __forceinline__ bool mean_free(const RParams& p) { return p.initial[3] > 0.0f; }
__device__ __forceinline__ bool pinned(const RView& s, uint32_t i) {
    return !mean_free(s.p) && (s.mask[i] & 3u) == 2u;
}
__device__ float diagonal(const RView& s, I3 pos) {  // :60-64
    float d = 0.0f;
    for (int axis = 0; axis < 3; axis++)
        for (int sign = -1; sign <= 1; sign += 2) {
            I3 q = pos;
            q.v[axis] += sign;
            if (fluid(s, q)) {
                I3 fp = pos;
                if (sign > 0) fp.v[axis] += 1;
                d += mobility(s, fp, axis);
            }
        }
    if (pinned(s, idx3(pos, s.p.dims))) return 1.0f;
    return fmaxf(d, 1e-30f);
}
__device__ float laplacian(const RView& s, I3 pos, int kind) {  // :65-69
    const float center = potential(s, pos, kind);
    float out = 0.0f;
    for (int axis = 0; axis < 3; axis++)
        for (int sign = -1; sign <= 1; sign += 2) {
            I3 q = pos;
            q.v[axis] += sign;
            if (fluid(s, q)) {
                I3 fp = pos;
                if (sign > 0) fp.v[axis] += 1;
                out += mobility(s, fp, axis) * (center - potential(s, q, kind));
            }
        }
    return out;
}
// cached_mobility: the cache holds the low faces at cell positions; a face at
// a non-periodic high boundary is a closed wall (0).
__device__ __forceinline__ float cached_mobility(const RView& s, I3 fp, int axis) {
    const I3 q = wrap_cell(s.p, fp);
    if (q.v[axis] >= (int)s.p.dims[axis]) return 0.0f;
    for (int a = 0; a < 3; a++)
        if (q.v[a] < 0 || q.v[a] >= (int)s.p.dims[a]) return 0.0f;
    const float4 c = s.cache[idx3(q, s.p.dims)];
    return axis == 0 ? c.x : (axis == 1 ? c.y : c.z);
}
__device__ float apply_cached(const RView& s, I3 pos, int kind) {  // :78-92
    if (pinned(s, idx3(pos, s.p.dims))) return potential(s, pos, kind);
    const float center = potential(s, pos, kind);
    float out = 0.0f;
    for (int axis = 0; axis < 3; axis++)
        for (int sign = -1; sign <= 1; sign += 2) {
            I3 fp = pos;
            if (sign > 0) fp.v[axis] += 1;
            const float beta = cached_mobility(s, fp, axis);
            if (beta > 0.0f) {
                I3 q = pos;
                q.v[axis] += sign;
                const float4 v = s.work[idx3(wrap_cell(s.p, q), s.p.dims)];
                out += beta * (center - (kind == 1 ? v.z : v.x));
            }
        }
    return out;
}
__device__ float divergence_star(const RView& s, I3 pos) {  // :104-106
    float sum = 0.0f;
    for (int axis = 0; axis < 3; axis++) {
        I3 q = pos;
        q.v[axis] += 1;
        sum += face_star(s, q, axis) - face_star(s, pos, axis);
    }
    return sum / s.p.physical[0];
}
__device__ float rhs(const RView& s, I3 pos) {  // :107
    if (pinned(s, idx3(pos, s.p.dims))) return 0.0f;
    return -s.p.physical[0] * s.p.physical[0] * divergence_star(s, pos);
}
__device__ float old_potential(const RView& s, I3 pos) {  // :164-167
    const I3 q = wrap_cell(s.p, pos);
    if (!fluid(s, q)) return 0.0f;
    const uint32_t i = idx3(q, s.p.dims), anchor = s.mask[i] >> 2u;
    return (s.oldp[i] - s.oldp[anchor]) * s.p.physical[1] / s.p.physical[3];
}

// --------------------------------------------------------- reductions
__device__ __forceinline__ void f4add(float4& a, const float4& b) {
    a.x += b.x;
    a.y += b.y;
    a.z += b.z;
    a.w += b.w;
}
// sum_group (solver.wgsl:118-120): the 256-lane tree.
__device__ __forceinline__ float4 tree256(float4* red, int l) {
    __syncthreads();
    for (int stride = 128; stride > 0; stride /= 2) {
        if (l < stride) f4add(red[l], red[l + stride]);
        __syncthreads();
    }
    return red[0];
}
// The single-workgroup second stage (initial_reduce etc., :199-203).
__device__ __forceinline__ float4 reduce_partials(const float4* partials, uint32_t groups, float4* red, int l) {
    float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
    for (uint32_t i = (uint32_t)l; i < groups; i += WG) f4add(sum, partials[i]);
    red[l] = sum;
    return tree256(red, l);
}
__device__ __forceinline__ uint32_t ngroups(const RParams& p) { return (p.dims[3] + 255u) / 256u; }
__device__ __forceinline__ bool converged(const RView& s) { return s.scalars[1].z >= 0.5f; }

// ------------------------------------------------------------ kernels
// pressure_coefficients (:93-103) at cell positions.
__global__ void kr_coefficients(RView s) {
    const uint32_t i = blockIdx.x * WG + threadIdx.x;
    if (i >= s.p.dims[3]) return;
    const I3 pos = decode3(i, s.p.dims);
    float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
    if (open_face(s, pos, 0)) c.x = mobility(s, pos, 0);
    if (open_face(s, pos, 1)) c.y = mobility(s, pos, 1);
    if (open_face(s, pos, 2)) c.z = mobility(s, pos, 2);
    if (s.mask[i] != 0u) c.w = diagonal(s, pos);
    s.cache[i] = c;
}
__global__ void kr_apply_probe(RView s, float* out) {
    const uint32_t i = blockIdx.x * WG + threadIdx.x;
    if (i >= s.p.dims[3]) return;
    out[i] = s.mask[i] != 0u ? apply_cached(s, decode3(i, s.p.dims), 1) : 0.0f;
}
// pressure_warm (:170-176), one thread per face of one axis.
__global__ void kr_warm(RView s, int axis, const float* us, float* pred) {
    const RParams& p = s.p;
    uint32_t d[3] = {p.dims[0], p.dims[1], p.dims[2]};
    d[axis] += 1;
    const uint32_t n = d[0] * d[1] * d[2];
    const uint32_t f = blockIdx.x * WG + threadIdx.x;
    if (f >= n) return;
    I3 pos;
    pos.v[0] = (int)(f % d[0]);
    pos.v[1] = (int)((f / d[0]) % d[1]);
    pos.v[2] = (int)(f / (d[0] * d[1]));
    float out = us[f];
    if (open_face(s, pos, axis)) {
        I3 left = pos;
        left.v[axis] -= 1;
        out -= mobility(s, pos, axis) * (old_potential(s, pos) - old_potential(s, left)) / p.physical[0];
    }
    pred[f] = out;
}
// pressure_guess (:177-180)
__global__ void kr_guess(RView s) {
    const uint32_t i = blockIdx.x * WG + threadIdx.x;
    if (i < s.p.dims[3]) s.work[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (i == 0u) {
        s.scalars[1].w = 0.0f;
        s.scalars[2].x = mean_free(s.p) ? 1.0f : 0.0f;
    }
}
// pressure_commit (:181-184)
__global__ void kr_commit(RView s) {
    const uint32_t i = blockIdx.x * WG + threadIdx.x;
    if (i < s.p.dims[3] && s.mask[i] != 0u) s.work[i].x += old_potential(s, decode3(i, s.p.dims));
}
// pressure_refresh (:185-197)
__global__ void kr_refresh(RView s) {
    __shared__ float4 red[WG];
    const int l = threadIdx.x;
    const uint32_t i = blockIdx.x * WG + l;
    float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
    if (i < s.p.dims[3] && s.mask[i] != 0u) {
        const I3 pos = decode3(i, s.p.dims);
        const float b = rhs(s, pos), r = b - apply_cached(s, pos, 0), d = s.cache[i].w;
        s.work[i].y = r;
        s.work[i].z = r / d;
        const float physical = -s.p.physical[0] * s.p.physical[0] * divergence_star(s, pos);
        const float true_residual = physical - laplacian(s, pos, 0);
        sum = make_float4(r * r / d, true_residual * true_residual, physical * physical,
                          mean_free(s.p) ? r : 0.0f);
    }
    red[l] = sum;
    const float4 total = tree256(red, l);
    if (l == 0) s.partials[blockIdx.x] = total;
}
// initial_reduce (:198-203)
__global__ void kr_initial_reduce(RView s) {
    __shared__ float4 red[WG];
    const int l = threadIdx.x;
    const float4 total = reduce_partials(s.partials, ngroups(s.p), red, l);
    if (l == 0) {
        s.scalars[0] = total;
        const bool flag = total.y <= s.p.solve[0] * total.z + s.p.solve[1] || total.z == 0.0f;
        s.scalars[1] = make_float4(0.0f, 0.0f, flag ? 1.0f : 0.0f, s.scalars[1].w);
    }
}
// pressure_apply (:204-210)
__global__ void kr_apply(RView s) {
    __shared__ float4 red[WG];
    const int l = threadIdx.x;
    const uint32_t i = blockIdx.x * WG + l;
    float value = 0.0f;
    if (i < s.p.dims[3] && s.mask[i] != 0u && !converged(s)) {
        const float a = apply_cached(s, decode3(i, s.p.dims), 1);
        s.work[i].w = a;
        value = s.work[i].z * a;
    }
    red[l] = make_float4(value, 0.f, 0.f, 0.f);
    const float4 total = tree256(red, l);
    if (l == 0) s.partials[blockIdx.x] = total;
}
// alpha_reduce (:211-215)
__global__ void kr_alpha_reduce(RView s) {
    __shared__ float4 red[WG];
    const int l = threadIdx.x;
    const float4 total = reduce_partials(s.partials, ngroups(s.p), red, l);
    if (l == 0) {
        float alpha = 0.0f;
        if (!converged(s)) alpha = s.scalars[0].x / fmaxf(total.x, 1e-35f);
        s.scalars[1].x = alpha;
    }
}
// update (:216-230)
__global__ void kr_update(RView s) {
    __shared__ float4 red[WG];
    const int l = threadIdx.x;
    const uint32_t i = blockIdx.x * WG + l;
    float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
    if (i < s.p.dims[3] && s.mask[i] != 0u && !converged(s)) {
        const float a = s.scalars[1].x;
        const float4 v = s.work[i];
        const float r = v.y - a * v.w;
        const float diag = s.cache[i].w;
        if (mean_free(s.p)) {
            // Search lanes stay read-only across invocations during this update.
            const float ref = s.work[s.mask[i] >> 2u].z;
            s.work[i].x = v.x + a * (v.z - ref);
            s.work[i].y = r;
            s.work[i].w = diag;
        } else {
            s.work[i] = make_float4(v.x + a * v.z, r, v.z, diag);
        }
        sum = make_float4(r * r / diag, r * r, 0.0f, mean_free(s.p) ? r : 0.0f);
    }
    red[l] = sum;
    const float4 total = tree256(red, l);
    if (l == 0) s.partials[blockIdx.x] = total;
}
// beta_reduce (:231-239)
__global__ void kr_beta_reduce(RView s) {
    __shared__ float4 red[WG];
    const int l = threadIdx.x;
    const float4 total = reduce_partials(s.partials, ngroups(s.p), red, l);
    if (l == 0 && !converged(s)) {
        s.scalars[1].w += 1.0f;
        s.scalars[1].y = total.x / fmaxf(s.scalars[0].x, 1e-35f);
        s.scalars[0].x = total.x;
        s.scalars[0].y = total.y;
        s.scalars[1].z = total.y <= (s.p.solve[0] * s.scalars[0].z + s.p.solve[1]) / s.p.solve[2] ? 1.0f : 0.0f;
    }
}
// search (:240-244)
__global__ void kr_search(RView s) {
    const uint32_t i = blockIdx.x * WG + threadIdx.x;
    if (i >= s.p.dims[3] || s.mask[i] == 0u || s.scalars[1].z > 0.5f) return;
    const float4 v = s.work[i];
    s.work[i].z = v.y / v.w + s.scalars[1].y * v.z;
}
// pressure_residual_mean (pressure_subspace.wgsl:3-7)
__global__ void kr_residual_mean(RView s) {
    __shared__ float4 red[WG];
    const int l = threadIdx.x;
    float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
    for (uint32_t i = (uint32_t)l; i < ngroups(s.p); i += WG) sum.x += s.partials[i].w;
    red[l] = sum;
    const float4 total = tree256(red, l);
    if (l == 0) s.scalars[2].y = total.x * s.p.initial[3];
}
// project_pressure_residual (pressure_subspace.wgsl:8-20)
__global__ void kr_project_residual(RView s, int initial) {
    __shared__ float4 red[WG];
    const int l = threadIdx.x;
    const uint32_t i = blockIdx.x * WG + l;
    float4 value = make_float4(0.f, 0.f, 0.f, 0.f);
    if (i < s.p.dims[3] && s.mask[i] != 0u && (initial || s.scalars[1].z < 0.5f)) {
        const float r = s.work[i].y - s.scalars[2].y;
        const float d = s.cache[i].w;
        s.work[i].y = r;
        if (initial) s.work[i].z = r / d;
        value = make_float4(r * r / d, r * r, 0.f, 0.f);
    }
    red[l] = value;
    const float4 total = tree256(red, l);
    if (l == 0) {
        const float4 old = s.partials[blockIdx.x];
        s.partials[blockIdx.x] = make_float4(total.x, initial ? old.y : total.y, old.z, 0.0f);
    }
}
// pressure_check / check_reduce (:317-328)
__global__ void kr_check(RView s) {
    __shared__ float4 red[WG];
    const int l = threadIdx.x;
    const uint32_t i = blockIdx.x * WG + l;
    float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
    if (i < s.p.dims[3] && s.mask[i] != 0u) {
        const I3 pos = decode3(i, s.p.dims);
        const float b = -s.p.physical[0] * s.p.physical[0] * divergence_star(s, pos);
        const float r = b - laplacian(s, pos, 0);
        sum.y = r * r;
    }
    red[l] = sum;
    const float4 total = tree256(red, l);
    if (l == 0) s.partials[blockIdx.x] = total;
}
__global__ void kr_check_reduce(RView s) {
    __shared__ float4 red[WG];
    const int l = threadIdx.x;
    const float4 total = reduce_partials(s.partials, ngroups(s.p), red, l);
    if (l == 0) {
        s.scalars[0].y = total.y;
        s.scalars[1].z = total.y <= s.p.solve[0] * s.scalars[0].z + s.p.solve[1] ? 1.0f : 0.0f;
    }
}
// correct (:245-250), one thread per face of one axis.  A periodic duplicate
// face carries the value of its canonical face.
__global__ void kr_correct(RView s, int axis, float* out) {
    const RParams& p = s.p;
    uint32_t d[3] = {p.dims[0], p.dims[1], p.dims[2]};
    d[axis] += 1;
    const uint32_t n = d[0] * d[1] * d[2];
    const uint32_t f = blockIdx.x * WG + threadIdx.x;
    if (f >= n) return;
    I3 pos;
    pos.v[0] = (int)(f % d[0]);
    pos.v[1] = (int)((f / d[0]) % d[1]);
    pos.v[2] = (int)(f / (d[0] * d[1]));
    float v = 0.0f;
    if (open_face(s, pos, axis)) {
        I3 left = pos;
        left.v[axis] -= 1;
        v = face_star(s, pos, axis) -
            mobility(s, pos, axis) * (potential(s, pos, 0) - potential(s, left, 0)) / p.physical[0];
    }
    out[f] = v;
}
// The pressure written by fields (:269-270): potential (minus the gauge cell in
// mean-free mode) * rho_l / dt.
__global__ void kr_pressure(RView s, float* out, float* keep) {
    const uint32_t i = blockIdx.x * WG + threadIdx.x;
    if (i >= s.p.dims[3]) return;
    float pr = 0.0f;
    if (s.mask[i] != 0u) {
        const float x = s.work[i].x;
        const float pot = mean_free(s.p) ? x - s.work[s.mask[i] >> 2u].x : x;
        pr = pot * s.p.physical[3] / s.p.physical[1];
    }
    if (out) out[i] = pr;
    keep[i] = pr;
}

// ------------------------------------------------ multigrid.wgsl kernels
struct Level {
    uint32_t dims[4], child[4], faces[4], location[4];
};
struct MView {
    Level L;
    const uint32_t* mask;
    const float4* cache;
    float4* work;
    float* temp;  // predicted.w lane
    float4* coeff;
    float4* value;
    float4* partials;
    const float4* scalars;
};
__device__ __forceinline__ bool mg_converged(const MView& m) { return m.scalars[1].z > 0.5f; }
__device__ __forceinline__ bool mg_meanfree(const MView& m) { return m.scalars[2].x > 0.5f; }
__device__ __forceinline__ I3 mg_canonical(const MView& m, I3 q, const uint32_t* d) {
    for (int a = 0; a < 3; a++)
        if (m.L.location[3] & (1u << a)) q.v[a] = wrap_periodic(q.v[a], d[a]);
    return q;
}
__device__ __forceinline__ bool mg_valid(I3 q, const uint32_t* d) {
    for (int a = 0; a < 3; a++)
        if (q.v[a] < 0 || q.v[a] >= (int)d[a]) return false;
    return true;
}
__device__ __forceinline__ bool fine_active(const MView& m, uint32_t i) {
    return m.mask[i] != 0u && (mg_meanfree(m) || (m.mask[i] & 3u) == 1u);
}
// edge() (:24-28); the fine cache reads the cell-indexed low-face record.
__device__ __forceinline__ float mg_edge(const MView& m, I3 q, int axis, int sign, const uint32_t* d, uint32_t offset,
                                         bool fine) {
    I3 f = q;
    if (sign > 0) f.v[axis] += 1;
    f = mg_canonical(m, f, d);
    if (fine) {
        if (f.v[axis] >= (int)d[axis]) return 0.0f;  // closed high boundary face
        const float4 c = m.cache[idx3(f, d)];
        return axis == 0 ? c.x : (axis == 1 ? c.y : c.z);
    }
    const float4 c = m.coeff[offset + idx3(f, d)];
    return axis == 0 ? c.x : (axis == 1 ? c.y : c.z);
}
__device__ __forceinline__ float mg_solution(const MView& m, uint32_t i, uint32_t offset, bool fine, bool temp) {
    if (fine) return temp ? m.temp[i] : m.work[i].w;
    const float4 v = m.value[offset + i];
    return temp ? v.z : v.y;
}
__device__ float mg_action(const MView& m, I3 q, const uint32_t* d, uint32_t offset, bool fine, bool temp) {  // :33-49
    const uint32_t i = idx3(q, d);
    const float center = mg_solution(m, i, offset, fine, temp);
    float out = 0.0f;
    if (fine) {
        for (int a = 0; a < 3; a++)
            for (int s = -1; s <= 1; s += 2) {
                const float beta = mg_edge(m, q, a, s, d, offset, true);
                if (beta > 0.0f) {
                    I3 n = q;
                    n.v[a] += s;
                    n = mg_canonical(m, n, d);
                    out += beta * (center - mg_solution(m, idx3(n, d), offset, true, temp));
                }
            }
        return out;
    }
    out = m.coeff[offset + i].w * center;
    for (int a = 0; a < 3; a++)
        for (int s = -1; s <= 1; s += 2) {
            I3 n = q;
            n.v[a] += s;
            n = mg_canonical(m, n, d);
            if (!mg_valid(n, d)) continue;
            const float beta = mg_edge(m, q, a, s, d, offset, false);
            if (beta > 0.0f) out += beta * (center - mg_solution(m, idx3(n, d), offset, false, temp));
        }
    return out;
}
// build (:50-65)
__global__ void kr_mg_build(MView m) {
    const Level& L = m.L;
    const uint32_t i = blockIdx.x * WG + threadIdx.x;
    if (i >= L.dims[3]) return;
    const I3 q = decode3(i, L.dims);
    float c[4] = {0.f, 0.f, 0.f, 0.f};
    float diag = 0.0f;
    const bool fine = L.location[2] == 1u;
    for (int z = 0; z < 2; z++)
        for (int y = 0; y < 2; y++)
            for (int x = 0; x < 2; x++) {
                I3 child;
                child.v[0] = 2 * q.v[0] + x;
                child.v[1] = 2 * q.v[1] + y;
                child.v[2] = 2 * q.v[2] + z;
                if (!mg_valid(child, L.child)) continue;
                const uint32_t ci = idx3(child, L.child);
                if (fine) {
                    if (!fine_active(m, ci)) continue;
                } else {
                    const float gamma = m.coeff[L.location[1] + ci].w;
                    c[3] += gamma;
                    diag += gamma;
                }
                for (int a = 0; a < 3; a++)
                    for (int s = -1; s <= 1; s += 2) {
                        I3 n = child;
                        n.v[a] += s;
                        n = mg_canonical(m, n, L.child);
                        if (!mg_valid(n, L.child)) continue;
                        const float beta = mg_edge(m, child, a, s, L.child, L.location[1], fine);
                        if (beta == 0.0f) continue;
                        if (fine && !mg_meanfree(m) && (m.mask[idx3(n, L.child)] & 3u) == 2u) {
                            c[3] += beta;
                            diag += beta;
                            continue;
                        }
                        if (n.v[0] / 2 == q.v[0] && n.v[1] / 2 == q.v[1] && n.v[2] / 2 == q.v[2]) continue;
                        diag += beta;
                        if (s < 0) c[a] += beta;
                    }
            }
    m.coeff[L.location[0] + i] = make_float4(c[0], c[1], c[2], c[3]);
    m.value[L.location[0] + i] = make_float4(0.f, 0.f, 0.f, diag);
}
// jacobi_step (:66-71); temp = false is smooth_to_temp.
__global__ void kr_mg_jacobi(MView m, int temp) {
    if (mg_converged(m)) return;
    const Level& L = m.L;
    const uint32_t i = blockIdx.x * WG + threadIdx.x;
    if (i >= L.dims[3]) return;
    const bool fine = L.location[2] == 0u;
    const uint32_t off = L.location[0];
    const I3 q = decode3(i, L.dims);
    float d, r;
    if (fine) {
        d = m.cache[i].w;
        r = m.work[i].y;
        if (!fine_active(m, i)) d = 0.0f;
    } else {
        d = m.value[off + i].w;
        r = m.value[off + i].x;
    }
    float next = 0.0f;
    if (d > 0.0f)
        next = mg_solution(m, i, off, fine, temp) + (2.0f / 3.0f) * (r - mg_action(m, q, L.dims, off, fine, temp)) / d;
    if (fine) {
        if (temp) m.work[i].w = next;
        else m.temp[i] = next;
    } else {
        if (temp) m.value[off + i].y = next;
        else m.value[off + i].z = next;
    }
}
// restrict_residual (:74-83)
__global__ void kr_mg_restrict(MView m) {
    if (mg_converged(m)) return;
    const Level& L = m.L;
    const uint32_t i = blockIdx.x * WG + threadIdx.x;
    if (i >= L.dims[3]) return;
    const I3 q = decode3(i, L.dims);
    const bool fine = L.location[2] == 1u;
    float sum = 0.0f;
    for (int z = 0; z < 2; z++)
        for (int y = 0; y < 2; y++)
            for (int x = 0; x < 2; x++) {
                I3 child;
                child.v[0] = 2 * q.v[0] + x;
                child.v[1] = 2 * q.v[1] + y;
                child.v[2] = 2 * q.v[2] + z;
                if (!mg_valid(child, L.child)) continue;
                const uint32_t ci = idx3(child, L.child);
                float r;
                if (fine) {
                    if (!fine_active(m, ci)) continue;
                    r = m.work[ci].y;
                } else {
                    r = m.value[L.location[1] + ci].x;
                }
                sum += r - mg_action(m, child, L.child, L.location[1], fine, false);
            }
    float4& v = m.value[L.location[0] + i];
    v.x = sum;
    v.y = 0.0f;
    v.z = 0.0f;
}
// prolong (:84-88)
__global__ void kr_mg_prolong(MView m) {
    if (mg_converged(m)) return;
    const Level& L = m.L;
    const uint32_t i = blockIdx.x * WG + threadIdx.x;
    if (i >= L.child[3]) return;
    const I3 q = decode3(i, L.child);
    I3 par;
    par.v[0] = q.v[0] / 2;
    par.v[1] = q.v[1] / 2;
    par.v[2] = q.v[2] / 2;
    const float correction = m.value[L.location[0] + idx3(par, L.dims)].y;
    if (L.location[2] == 1u) {
        if (fine_active(m, i)) m.work[i].w += correction;
    } else {
        m.value[L.location[1] + i].y += correction;
    }
}
// coarse_solve (:106-131): COARSE_SWEEPS Jacobi steps in one workgroup.
__global__ void kr_mg_coarse_solve(MView m) {
    if (mg_converged(m)) return;
    __shared__ float sol[WG];
    const Level& L = m.L;
    const int i = threadIdx.x;
    const bool fine = L.location[2] == 0u;
    const uint32_t off = L.location[0];
    const bool in_grid = (uint32_t)i < L.dims[3];
    float r = 0.f, diag = 0.f, reaction = 0.f;
    I3 q;
    q.v[0] = q.v[1] = q.v[2] = 0;
    if (in_grid) {
        q = decode3((uint32_t)i, L.dims);
        if (fine) {
            if (fine_active(m, (uint32_t)i)) {
                r = m.work[i].y;
                diag = m.cache[i].w;
            }
        } else {
            r = m.value[off + i].x;
            diag = m.value[off + i].w;
            reaction = m.coeff[off + i].w;
        }
    }
    sol[i] = 0.0f;
    __syncthreads();
    for (uint32_t step = 0; step < COARSE_SWEEPS; step++) {
        const float center = sol[i];
        float next = 0.0f;
        if (in_grid && diag > 0.0f) {
            float a = reaction * center;
            for (int axis = 0; axis < 3; axis++)
                for (int s = -1; s <= 1; s += 2) {
                    I3 n = q;
                    n.v[axis] += s;
                    n = mg_canonical(m, n, L.dims);
                    if (!mg_valid(n, L.dims)) continue;
                    const uint32_t ni = idx3(n, L.dims);
                    float neighbor = sol[ni];
                    if (fine && !fine_active(m, ni)) neighbor = 0.0f;
                    a += mg_edge(m, q, axis, s, L.dims, off, fine) * (center - neighbor);
                }
            next = center + (2.0f / 3.0f) * (r - a) / diag;
        }
        __syncthreads();
        sol[i] = next;
        __syncthreads();
    }
    if (in_grid) {
        if (fine) m.work[i].w = sol[i];
        else m.value[off + i].y = sol[i];
    }
}
// diagonal_start (:133-139)
__global__ void kr_mg_diagonal_start(MView m) {
    const Level& L = m.L;
    const uint32_t i = blockIdx.x * WG + threadIdx.x;
    if (i >= L.dims[3] || mg_converged(m)) return;
    float z = 0.0f;
    if (L.location[2] == 0u) {
        if (fine_active(m, i)) z = (2.0f / 3.0f) * m.work[i].y / m.cache[i].w;
        m.work[i].w = z;
    } else {
        float4& v = m.value[L.location[0] + i];
        if (v.w > 0.0f) z = (2.0f / 3.0f) * v.x / v.w;
        v.y = z;
    }
}
// commit_smooth (:140-144)
__global__ void kr_mg_commit(MView m) {
    const Level& L = m.L;
    const uint32_t i = blockIdx.x * WG + threadIdx.x;
    if (i >= L.dims[3] || mg_converged(m)) return;
    if (L.location[2] == 0u) m.work[i].w = m.temp[i];
    else m.value[L.location[0] + i].y = m.value[L.location[0] + i].z;
}
// dot_partial (:90-96): initial_direction / preconditioned_dot
__global__ void kr_mg_dot(MView m, int initial) {
    __shared__ float4 red[WG];
    const Level& L = m.L;
    const int l = threadIdx.x;
    const uint32_t i = blockIdx.x * WG + l;
    const bool conv = mg_converged(m);
    float v = 0.0f;
    if (i < L.dims[3] && fine_active(m, i) && !conv) {
        v = m.work[i].y * m.work[i].w;
        if (initial) m.work[i].z = m.work[i].w;
    }
    red[l] = make_float4(v, 0.f, 0.f, 0.f);
    const float4 total = tree256(red, l);
    if (l == 0 && !conv) m.partials[blockIdx.x].x = total.x;
}
// preconditioned_search (:101-102)
__global__ void kr_mg_search(MView m) {
    const Level& L = m.L;
    const uint32_t i = blockIdx.x * WG + threadIdx.x;
    if (i >= L.dims[3] || !fine_active(m, i) || mg_converged(m)) return;
    m.work[i].z = m.work[i].w + m.scalars[1].y * m.work[i].z;
}
}  // namespace

// --------------------------------------------------------------- state
struct RefState {
    mhdproj_grid grid{};
    mhdproj_options opt{};
    cudaStream_t stream = nullptr;
    RParams p{};
    uint32_t n = 0, groups = 0;
    uint32_t components = 0, fluid_cells = 0;
    bool have_topology = false, have_coef = false, have_pressure = false;
    // device
    uint32_t* mask = nullptr;
    float* occ = nullptr;
    float* phase = nullptr;
    float* oldp = nullptr;
    float* pred[3] = {nullptr, nullptr, nullptr};
    float4* cache = nullptr;
    float4* work = nullptr;
    float* temp = nullptr;
    float4* partials = nullptr;
    float4* scalars = nullptr;
    float4* h_scalars = nullptr;
    // multigrid
    std::vector<Level> levels;
    uint64_t coarse_cells = 0;
    float4* coeff = nullptr;
    float4* value = nullptr;
    bool mg_ready = false;
    float drag_rate = 1e6f, drag_dt = 1e-5f;
    bool drag = false;
    std::vector<void*> allocs;
};

#define RCK(call)                                                                 \
    do {                                                                          \
        cudaError_t _e = (call);                                                  \
        if (_e != cudaSuccess) {                                                  \
            err = std::string(#call ": ") + cudaGetErrorString(_e);               \
            return _e == cudaErrorMemoryAllocation ? MHDPROJ_ERR_OUT_OF_MEMORY : MHDPROJ_ERR_CUDA; \
        }                                                                         \
    } while (0)

template <class T>
static cudaError_t ralloc(RefState* s, T** p, size_t bytes) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, bytes ? bytes : 16);
    if (e != cudaSuccess) return e;
    s->allocs.push_back(q);
    *p = (T*)q;
    return cudaMemsetAsync(q, 0, bytes ? bytes : 16, s->stream);
}

static RView view(RefState* s, const float* const us[3]) {
    RView v;
    v.p = s->p;
    v.mask = s->mask;
    v.occ = s->occ;
    v.phase = s->phase;
    v.oldp = s->oldp;
    for (int a = 0; a < 3; a++) v.us[a] = us ? us[a] : nullptr;
    v.cache = s->cache;
    v.work = s->work;
    v.partials = s->partials;
    v.scalars = s->scalars;
    return v;
}
static MView mview(RefState* s, int level) {
    MView m;
    m.L = s->levels[level];
    m.mask = s->mask;
    m.cache = s->cache;
    m.work = s->work;
    m.temp = s->temp;
    m.coeff = s->coeff;
    m.value = s->value;
    m.partials = s->partials;
    m.scalars = s->scalars;
    return m;
}
static unsigned blocks_for(uint32_t n) { return (n + WG - 1) / WG; }

int ref_create(RefState** out, const mhdproj_grid* grid, const mhdproj_options* opt, cudaStream_t stream,
               std::string& err) {
    RefState* s = new RefState();
    s->grid = *grid;
    s->opt = *opt;
    s->stream = stream;
    s->n = grid->nx * grid->ny * grid->nz;
    s->groups = (s->n + 255u) / 256u;
    *out = s;
    const size_t n = s->n;
    RCK(ralloc(s, &s->mask, n * 4));
    RCK(ralloc(s, &s->occ, n * 4));
    RCK(ralloc(s, &s->phase, n * 4));
    RCK(ralloc(s, &s->oldp, n * 4));
    const size_t nf[3] = {(size_t)(grid->nx + 1) * grid->ny * grid->nz, (size_t)grid->nx * (grid->ny + 1) * grid->nz,
                          (size_t)grid->nx * grid->ny * (grid->nz + 1)};
    for (int a = 0; a < 3; a++) RCK(ralloc(s, &s->pred[a], nf[a] * 4));
    RCK(ralloc(s, &s->cache, n * sizeof(float4)));
    RCK(ralloc(s, &s->work, n * sizeof(float4)));
    RCK(ralloc(s, &s->temp, n * 4));
    RCK(ralloc(s, &s->partials, (size_t)s->groups * sizeof(float4)));
    RCK(ralloc(s, &s->scalars, 5 * sizeof(float4)));
    RCK(cudaMallocHost(&s->h_scalars, 5 * sizeof(float4)));
    // hierarchy() (multigrid.rs:25-65); allocated lazily at the first
    // multigrid solve as the reference does
    const uint32_t dims[4] = {grid->nx, grid->ny, grid->nz, (uint32_t)n};
    uint32_t nl = 0;
    uint64_t cc = 0;
    if (host_hierarchy(dims, &nl, &cc) == 0) {
        Level L0{};
        for (int a = 0; a < 3; a++) {
            L0.dims[a] = dims[a];
            L0.child[a] = dims[a];
            L0.faces[a] = dims[a] + 1;
        }
        L0.dims[3] = L0.child[3] = dims[3];
        L0.faces[3] = L0.faces[0] * L0.faces[1] * L0.faces[2];
        L0.location[3] = grid->periodic;
        s->levels.push_back(L0);
        uint32_t offset = 0;
        while (s->levels.back().dims[0] > 4 || s->levels.back().dims[1] > 4 || s->levels.back().dims[2] > 4) {
            const Level& C = s->levels.back();
            Level L{};
            for (int a = 0; a < 3; a++) L.dims[a] = (C.dims[a] + 1) / 2;
            L.dims[3] = L.dims[0] * L.dims[1] * L.dims[2];
            for (int a = 0; a < 4; a++) {
                L.child[a] = C.dims[a];
                L.faces[a] = L0.faces[a];
            }
            L.location[0] = offset;
            L.location[1] = C.location[0];
            L.location[2] = (uint32_t)s->levels.size();
            L.location[3] = grid->periodic;
            offset += L.dims[3];
            s->levels.push_back(L);
        }
        s->coarse_cells = cc;
    }
    return 0;
}

void ref_destroy(RefState* s) {
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (void* p : s->allocs) cudaFree(p);
    if (s->h_scalars) cudaFreeHost(s->h_scalars);
    delete s;
}
void ref_set_stream(RefState* s, cudaStream_t stream) { s->stream = stream; }

// FluidState::new's Params and configure_pressure_projection.
static void make_params(RefState* s, float rho_l, float rho_air) {
    RParams& p = s->p;
    memset(&p, 0, sizeof p);
    const mhdproj_grid& g = s->grid;
    p.dims[0] = g.nx;
    p.dims[1] = g.ny;
    p.dims[2] = g.nz;
    p.dims[3] = s->n;
    for (int a = 0; a < 3; a++) p.faces[a] = p.dims[a] + 1;
    p.faces[3] = p.faces[0] * p.faces[1] * p.faces[2];
    p.flags[0] = g.periodic;
    p.flags[3] = s->drag ? 1u : 0u;
    p.physical[0] = g.h;
    p.physical[1] = s->drag_dt;
    p.physical[3] = rho_l;
    p.surface[0] = s->opt.two_phase ? 1.0f : 0.0f;
    p.surface[1] = s->opt.two_phase ? rho_air : rho_l;
    const float tol = s->opt.rel_tol, at = s->opt.abs_div_tol, h2 = g.h * g.h;
    p.solve[0] = tol * tol;
    p.solve[1] = (at * at) * (h2 * h2) * (float)s->fluid_cells;
    p.solve[3] = s->drag_rate;
    bool meanfree = s->components == 1u;
    if (s->opt.gauge >= 0) meanfree = s->opt.gauge == 1 && s->components == 1u;
    const uint32_t nf = s->fluid_cells ? s->fluid_cells : 1u;
    p.initial[3] = meanfree ? 1.0f / (float)nf : 0.0f;
    p.solve[2] = meanfree ? 1.0f : (float)nf;
}

int ref_set_topology(RefState* s, const uint32_t* mask_host, uint32_t components, std::string& err) {
    RCK(cudaMemcpyAsync(s->mask, mask_host, (size_t)s->n * 4, cudaMemcpyHostToDevice, s->stream));
    uint32_t nf = 0;
    for (uint32_t i = 0; i < s->n; i++) nf += mask_host[i] != 0u;
    s->fluid_cells = nf;
    s->components = components;
    s->have_topology = true;
    RCK(cudaStreamSynchronize(s->stream));
    return 0;
}

uint32_t* ref_mask(RefState* s) { return s->mask; }

RefExport ref_export(RefState* s) {
    RefExport e{};
    e.mask = s->mask;
    e.occ = s->occ;
    e.phase = s->drag ? s->phase : nullptr;
    e.work = reinterpret_cast<const float*>(s->work);
    e.fluid_cells = s->fluid_cells;
    e.mean_free = s->p.initial[3] > 0.0f;
    e.two_phase = s->p.surface[0] > 0.5f;
    e.rho_l = s->p.physical[3];
    e.rho_air = s->p.surface[1];
    e.drag_rate = s->drag_rate;
    e.drag_dt = s->drag_dt;
    return e;
}

void ref_set_topology_device(RefState* s, uint32_t components, uint32_t fluid_cells) {
    s->fluid_cells = fluid_cells;
    s->components = components;
    s->have_topology = true;
}

int ref_set_phase_drag(RefState* s, const float* phase, float drag_rate, float dt, std::string& err) {
    if (!phase) {
        s->drag = false;
        s->p.flags[3] = 0u;
        return 0;
    }
    if (!(drag_rate > 0.0f) || !(dt > 0.0f)) {
        err = "Invalid fluid timestep, initial condition or solver limits/tolerances";
        return MHDPROJ_ERR_INVALID;
    }
    RCK(cudaMemcpyAsync(s->phase, phase, (size_t)s->n * 4, cudaMemcpyDeviceToDevice, s->stream));
    s->drag = true;
    s->drag_rate = drag_rate;
    s->drag_dt = dt;
    s->p.flags[3] = 1u;
    s->p.solve[3] = drag_rate;
    s->p.physical[1] = dt;
    return 0;
}

int ref_set_coefficients(RefState* s, const float* alpha, float rho_l, float rho_air, std::string& err) {
    RCK(cudaMemcpyAsync(s->occ, alpha, (size_t)s->n * 4, cudaMemcpyDeviceToDevice, s->stream));
    make_params(s, rho_l, rho_air);
    s->have_coef = true;
    return 0;
}

// Rust's {:.3e}: three decimals, exponent without sign padding ("1.234e-3").
static std::string rust_sci(double v) {
    char buf[64];
    snprintf(buf, sizeof buf, "%.3e", v);
    std::string s(buf);
    const size_t e = s.find('e');
    if (e == std::string::npos) return s;  // inf / nan
    const std::string mant = s.substr(0, e);
    int exp = atoi(s.c_str() + e + 1);
    return mant + "e" + std::to_string(exp);
}

// convergence() (src/fluid/mod.rs:969-977)
static int read_convergence(RefState* s, float* residual, bool* conv, uint32_t* its, std::string& err) {
    RCK(cudaMemcpyAsync(s->h_scalars, s->scalars, 2 * sizeof(float4), cudaMemcpyDeviceToHost, s->stream));
    RCK(cudaStreamSynchronize(s->stream));
    const float* f = reinterpret_cast<const float*>(s->h_scalars);
    const float r = std::sqrt(f[1] / std::fmax(f[2], 1e-38f));
    bool bad = !std::isfinite(r) || f[1] < 0.0f || f[2] < 0.0f;
    for (int k = 0; k < 8; k++)
        if (!std::isfinite(f[k])) bad = true;
    if (bad) {
        err = "Nonfinite fluid pressure residual";
        return MHDPROJ_ERR_NONFINITE;
    }
    *residual = r;
    *conv = f[6] > 0.5f;
    *its = (uint32_t)f[7];
    return 0;
}

static void refresh_stages(RefState* s, const RView& v) {  // pressure_refresh_stages (:1003-1014)
    kr_refresh<<<s->groups, WG, 0, s->stream>>>(v);
    if (s->p.initial[3] > 0.0f) {
        kr_residual_mean<<<1, WG, 0, s->stream>>>(v);
        kr_project_residual<<<s->groups, WG, 0, s->stream>>>(v, 1);
    }
    kr_initial_reduce<<<1, WG, 0, s->stream>>>(v);
}
static void mg_cycle(RefState* s) {  // cycle_stages (multigrid.rs:67-82)
    const int L = (int)s->levels.size();
    for (int l = 0; l + 1 < L; l++) {
        kr_mg_diagonal_start<<<blocks_for(s->levels[l].dims[3]), WG, 0, s->stream>>>(mview(s, l));
        kr_mg_restrict<<<blocks_for(s->levels[l + 1].dims[3]), WG, 0, s->stream>>>(mview(s, l + 1));
    }
    kr_mg_coarse_solve<<<1, WG, 0, s->stream>>>(mview(s, L - 1));
    for (int l = L - 2; l >= 0; l--) {
        kr_mg_prolong<<<blocks_for(s->levels[l + 1].child[3]), WG, 0, s->stream>>>(mview(s, l + 1));
        kr_mg_jacobi<<<blocks_for(s->levels[l].dims[3]), WG, 0, s->stream>>>(mview(s, l), 0);
        kr_mg_commit<<<blocks_for(s->levels[l].dims[3]), WG, 0, s->stream>>>(mview(s, l));
    }
}
static void mg_initialize(RefState* s, const RView& v) {  // multigrid.rs:287-291
    mg_cycle(s);
    kr_mg_dot<<<s->groups, WG, 0, s->stream>>>(mview(s, 0), 1);
    kr_initial_reduce<<<1, WG, 0, s->stream>>>(v);
}
static void mg_iterate(RefState* s, const RView& v, uint32_t batch) {  // multigrid.rs:292-329
    const bool mf = s->p.initial[3] > 0.0f;
    for (uint32_t b = 0; b < batch; b++) {
        kr_apply<<<s->groups, WG, 0, s->stream>>>(v);
        kr_alpha_reduce<<<1, WG, 0, s->stream>>>(v);
        kr_update<<<s->groups, WG, 0, s->stream>>>(v);
        if (mf) {
            kr_residual_mean<<<1, WG, 0, s->stream>>>(v);
            kr_project_residual<<<s->groups, WG, 0, s->stream>>>(v, 0);
        }
        mg_cycle(s);
        kr_mg_dot<<<s->groups, WG, 0, s->stream>>>(mview(s, 0), 0);
        kr_beta_reduce<<<1, WG, 0, s->stream>>>(v);
        kr_mg_search<<<s->groups, WG, 0, s->stream>>>(mview(s, 0));
    }
}
static void jacobi_iterate(RefState* s, const RView& v, uint32_t batch) {  // mod.rs:1060-1075
    const bool mf = s->p.initial[3] > 0.0f;
    for (uint32_t b = 0; b < batch; b++) {
        kr_apply<<<s->groups, WG, 0, s->stream>>>(v);
        kr_alpha_reduce<<<1, WG, 0, s->stream>>>(v);
        kr_update<<<s->groups, WG, 0, s->stream>>>(v);
        if (mf) {
            kr_residual_mean<<<1, WG, 0, s->stream>>>(v);
            kr_project_residual<<<s->groups, WG, 0, s->stream>>>(v, 0);
        }
        kr_beta_reduce<<<1, WG, 0, s->stream>>>(v);
        kr_search<<<s->groups, WG, 0, s->stream>>>(v);
    }
}

// FluidState::project (src/fluid/mod.rs:1015-1115) + correct + fields pressure.
int ref_project(RefState* s, const float* us, const float* vs, const float* ws, float* uo, float* vo, float* wo,
                float* po, float dt, int warm, mhdproj_stats* st, std::string& err) {
    if (!s->have_topology || !s->have_coef) {
        err = "call mhdproj_set_coefficients before projecting";
        return MHDPROJ_ERR_STATE;
    }
    // physical.y is the timestep of the projection (it scales the pressure and
    // the warm-start potential); the drag term uses the same dt.
    if (!s->drag) s->p.physical[1] = dt;
    else if (dt != s->drag_dt) {
        err = "the phase-drag mobility was set for a different dt; call mhdproj_set_phase_drag again";
        return MHDPROJ_ERR_INVALID;
    }
    const float* in[3] = {us, vs, ws};
    const size_t nf[3] = {(size_t)(s->grid.nx + 1) * s->grid.ny * s->grid.nz,
                          (size_t)s->grid.nx * (s->grid.ny + 1) * s->grid.nz,
                          (size_t)s->grid.nx * s->grid.ny * (s->grid.nz + 1)};
    const float* star[3] = {us, vs, ws};
    const bool do_warm = warm != 0;
    if (do_warm) {
        RView v0 = view(s, in);
        for (int a = 0; a < 3; a++) {
            kr_warm<<<blocks_for((uint32_t)nf[a]), WG, 0, s->stream>>>(v0, a, in[a], s->pred[a]);
            star[a] = s->pred[a];
        }
    }
    RView v = view(s, star);
    kr_coefficients<<<blocks_for(s->n), WG, 0, s->stream>>>(v);
    kr_guess<<<blocks_for(s->n), WG, 0, s->stream>>>(v);
    refresh_stages(s, v);
    RCK(cudaGetLastError());
    uint32_t iterations = 0, it_read = 0;
    float residual = 0.0f;
    bool conv = false;
    int rc = read_convergence(s, &residual, &conv, &it_read, err);
    if (rc) return rc;
    bool preferred = s->n >= MIN_CELLS;
    if (s->opt.preconditioner == MHDPROJ_PRECOND_JACOBI) preferred = false;
    if (s->opt.preconditioner == MHDPROJ_PRECOND_MULTIGRID) preferred = true;
    bool mg = false;
    if (preferred && !conv && !s->levels.empty()) {
        if (!s->mg_ready) {
            // Multigrid::new (multigrid.rs:85-234): the optional workspace; a
            // failed allocation keeps Jacobi-CG (mod.rs:1035-1043).
            const size_t bytes = (size_t)(s->coarse_cells ? s->coarse_cells : 1) * sizeof(float4);
            if (ralloc(s, &s->coeff, bytes) == cudaSuccess && ralloc(s, &s->value, bytes) == cudaSuccess)
                s->mg_ready = true;
            else
                (void)cudaGetLastError();
        }
        mg = s->mg_ready;
    }
    if (!conv && mg) {
        for (size_t l = 1; l < s->levels.size(); l++)
            kr_mg_build<<<blocks_for(s->levels[l].dims[3]), WG, 0, s->stream>>>(mview(s, (int)l));
        mg_initialize(s, v);
    }
    const uint32_t max_it = s->opt.max_iterations;
    const bool mf = s->p.initial[3] > 0.0f;
    while (!conv && iterations < max_it) {
        uint32_t batch = mg ? 8u : 32u;
        batch = std::min(batch, max_it - iterations);
        batch = std::min(batch, 64u - iterations % 64u);
        if (mg) mg_iterate(s, v, batch);
        else jacobi_iterate(s, v, batch);
        RCK(cudaGetLastError());
        rc = read_convergence(s, &residual, &conv, &it_read, err);
        if (rc) return rc;
        if (it_read <= iterations && !conv) {
            err = "Fluid pressure iteration made no progress";
            return MHDPROJ_ERR_NO_PROGRESS;
        }
        iterations = it_read;
        if (conv) {
            refresh_stages(s, v);
            rc = read_convergence(s, &residual, &conv, &it_read, err);
            if (rc) return rc;
            if (!conv && mg) mg_initialize(s, v);
        } else if (iterations % 64u == 0u || iterations == max_it) {
            kr_check<<<s->groups, WG, 0, s->stream>>>(v);
            kr_check_reduce<<<1, WG, 0, s->stream>>>(v);
            rc = read_convergence(s, &residual, &conv, &it_read, err);
            if (rc) return rc;
        }
    }
    (void)mf;
    if (!conv) {
        err = "Fluid pressure solve did not converge after " + std::to_string(iterations) +
              " iterations (true relative residual " + rust_sci(residual) + ", requested " +
              rust_sci(s->opt.rel_tol) + ", RMS divergence floor " + rust_sci(s->opt.abs_div_tol) +
              " s\xe2\x81\xbb\xc2\xb9)";
        return MHDPROJ_ERR_NOT_CONVERGED;
    }
    float* outs[3] = {uo, vo, wo};
    for (int a = 0; a < 3; a++) kr_correct<<<blocks_for((uint32_t)nf[a]), WG, 0, s->stream>>>(v, a, outs[a]);
    if (do_warm) kr_commit<<<blocks_for(s->n), WG, 0, s->stream>>>(v);
    kr_pressure<<<blocks_for(s->n), WG, 0, s->stream>>>(v, po, s->oldp);
    RCK(cudaGetLastError());
    s->have_pressure = true;
    if (st) {
        st->iterations = iterations;
        st->refinements = 0;
        st->relative_residual = residual;
        st->true_relative_residual = residual;
        st->meanfree = s->p.initial[3] > 0.0f;
        st->multigrid = mg;
        st->levels = mg ? (uint32_t)s->levels.size() : 0u;
        st->coarse_cells = mg ? s->coarse_cells : 0u;
    }
    return 0;
}

int ref_apply_operator(RefState* s, const float* x, float* y, std::string& err) {
    // apply(pos, 1) on the cached coefficients with x in the search lane.
    RView v = view(s, nullptr);
    kr_coefficients<<<blocks_for(s->n), WG, 0, s->stream>>>(v);
    RCK(cudaMemcpy2DAsync(reinterpret_cast<char*>(s->work) + 8, sizeof(float4), x, sizeof(float), sizeof(float), s->n,
                          cudaMemcpyDeviceToDevice, s->stream));
    kr_apply_probe<<<blocks_for(s->n), WG, 0, s->stream>>>(v, y);
    RCK(cudaGetLastError());
    return 0;
}

int ref_apply_preconditioner(RefState* s, const float* r, float* z, std::string& err) {
    // The preconditioner of the projection's choice: the fixed aggregation
    // V-cycle (multigrid) or r / diag (Jacobi).
    RView v = view(s, nullptr);
    kr_coefficients<<<blocks_for(s->n), WG, 0, s->stream>>>(v);
    RCK(cudaMemsetAsync(s->work, 0, (size_t)s->n * sizeof(float4), s->stream));
    RCK(cudaMemcpy2DAsync(reinterpret_cast<char*>(s->work) + 4, sizeof(float4), r, sizeof(float), sizeof(float), s->n,
                          cudaMemcpyDeviceToDevice, s->stream));
    RCK(cudaMemsetAsync(s->scalars, 0, 5 * sizeof(float4), s->stream));
    {
        const float mfv = s->p.initial[3] > 0.0f ? 1.0f : 0.0f;
        RCK(cudaMemcpyAsync(reinterpret_cast<char*>(s->scalars) + 2 * sizeof(float4), &mfv, sizeof(float),
                            cudaMemcpyHostToDevice, s->stream));
    }
    bool preferred = s->n >= MIN_CELLS;
    if (s->opt.preconditioner == MHDPROJ_PRECOND_JACOBI) preferred = false;
    if (s->opt.preconditioner == MHDPROJ_PRECOND_MULTIGRID) preferred = true;
    if (preferred && !s->levels.empty()) {
        if (!s->mg_ready) {
            const size_t bytes = (size_t)(s->coarse_cells ? s->coarse_cells : 1) * sizeof(float4);
            RCK(ralloc(s, &s->coeff, bytes));
            RCK(ralloc(s, &s->value, bytes));
            s->mg_ready = true;
        }
        for (size_t l = 1; l < s->levels.size(); l++)
            kr_mg_build<<<blocks_for(s->levels[l].dims[3]), WG, 0, s->stream>>>(mview(s, (int)l));
        mg_cycle(s);
        RCK(cudaMemcpy2DAsync(z, sizeof(float), reinterpret_cast<char*>(s->work) + 12, sizeof(float4), sizeof(float),
                              s->n, cudaMemcpyDeviceToDevice, s->stream));
    } else {
        // z = r / diag on fluid cells (search after a zero direction)
        RCK(cudaMemcpy2DAsync(reinterpret_cast<char*>(s->work) + 12, sizeof(float4),
                              reinterpret_cast<char*>(s->cache) + 12, sizeof(float4), sizeof(float), s->n,
                              cudaMemcpyDeviceToDevice, s->stream));
        kr_search<<<blocks_for(s->n), WG, 0, s->stream>>>(v);
        RCK(cudaMemcpy2DAsync(z, sizeof(float), reinterpret_cast<char*>(s->work) + 8, sizeof(float4), sizeof(float),
                              s->n, cudaMemcpyDeviceToDevice, s->stream));
    }
    RCK(cudaGetLastError());
    return 0;
}

int ref_copy_coefficients(RefState* s, float* coef4, std::string& err) {
    RView v = view(s, nullptr);
    kr_coefficients<<<blocks_for(s->n), WG, 0, s->stream>>>(v);
    RCK(cudaMemcpyAsync(coef4, s->cache, (size_t)s->n * sizeof(float4), cudaMemcpyDeviceToDevice, s->stream));
    return 0;
}

__global__ static void kr_potential_double(const float4* work, double* out, uint32_t n) {
    const uint32_t i = blockIdx.x * WG + threadIdx.x;
    if (i < n) out[i] = (double)work[i].x;
}
int ref_copy_potential(RefState* s, double* phi, std::string& err) {
    kr_potential_double<<<blocks_for(s->n), WG, 0, s->stream>>>(s->work, phi, s->n);
    RCK(cudaGetLastError());
    return 0;
}


}  // namespace mhdproj
