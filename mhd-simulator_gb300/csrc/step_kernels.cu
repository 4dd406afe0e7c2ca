// step_kernels.cu -- the fluid step around the projection: semi-Lagrangian
// advection, explicit viscosity and forcing, and the per-cell fields and
// diagnostics reductions.
//
// Each kernel restates one WGSL entry point of src/fluid/solver.wgsl for a
// step without a moving interface (FluidState::step, src/fluid/mod.rs:
// 1246-1333):
//   ks_open_faces   face() and open_face() of every face position (zero
//                   where closed, periodic positions canonical), once per
//                   step;
//   ks_predict      predict (:127-141): u at the face, or with advection the
//                   value at the RK2 departure point, trilinear in the face
//                   grid of that axis, sampled from those arrays;
//   ks_viscous      viscous (:143-163): explicit 6-neighbour Laplacian
//                   (closed tangential neighbours mirrored: no slip), body and
//                   EM acceleration, times the face mobility; the open tests
//                   read the flags of ks_open_faces;
//   ks_fields       fields (:256-285): the 16-float cell record (velocity and
//                   speed, pressure and divergence, force, reserved) and the
//                   per-workgroup max/sum reductions;
//   ks_diagnostics  diagnostics (:286-291): the single-workgroup final pass.
// With a moving interface (two densities) viscous adds the capillary force
// with face densities, and the Newtonian stresses of src/fluid/viscosity.wgsl
// diffuse the predicted velocity first (diffuse_surface_stress,
// src/fluid/mod.rs:1160-1240):
//   ks_viscosity_bound(_edge)  the stability bound, max over faces;
//   ks_stress_coefficients     the cell viscosity of the step;
//   ks_stress_cells(_edge), ks_stress_ghosts, ks_stress_diffuse
//                              one explicit Euler substep;
//   ks_stress_tensor, ks_stress_save_initial, ks_stress_stage
//                              the damped RKC2 stages (stabilized.wgsl).
// Faces are the SoA arrays of include/mhdproj.h, one launch per axis.  The
// arithmetic keeps the reference's operation order without fused
// multiply-adds (this unit is compiled with -fmad=false) and the reductions
// replay the reference's 256-lane tree and 256-stride final pass, so results
// equal the oracle's restatement bit for bit.
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"

namespace mhdproj {

namespace {
constexpr int WG = 256;

struct P3 {
    int v[3];
};

__device__ __forceinline__ int32_t wrap_periodic(int32_t value, uint32_t size) {  // periodic.wgsl:5
    if (value >= 0) return (int32_t)((uint32_t)value % size);
    const uint32_t magnitude = (uint32_t)(-(value + 1)) + 1u;
    const uint32_t remainder = magnitude % size;
    return (int32_t)(remainder == 0u ? 0u : size - remainder);
}
__device__ __forceinline__ uint32_t cell_index(const StepView& s, P3 q) {
    return (uint32_t)q.v[0] + s.dims[0] * ((uint32_t)q.v[1] + s.dims[1] * (uint32_t)q.v[2]);
}
__device__ __forceinline__ P3 wrap_cell(const StepView& s, P3 q) {
    for (int a = 0; a < 3; a++)
        if (s.periodic & (1u << a)) q.v[a] = wrap_periodic(q.v[a], s.dims[a]);
    return q;
}
__device__ __forceinline__ bool valid_cell(const StepView& s, P3 q) {
    for (int a = 0; a < 3; a++)
        if (q.v[a] < 0 || q.v[a] >= (int)s.dims[a]) return false;
    return true;
}
__device__ __forceinline__ bool is_fluid_index(const StepView& s, uint32_t i) {
    return s.mask ? s.mask[i] != 0u : s.cls[i] != 0;
}
__device__ __forceinline__ bool fluid(const StepView& s, P3 pos) {
    const P3 q = wrap_cell(s, pos);
    if (!valid_cell(s, q)) return false;
    return is_fluid_index(s, cell_index(s, q));
}
__device__ __forceinline__ bool valid_face(const StepView& s, P3 q, int axis) {
    for (int a = 0; a < 3; a++) {
        const int lim = (int)s.dims[a] + (a == axis ? 1 : 0);
        if (q.v[a] < 0 || q.v[a] >= lim) return false;
    }
    return true;
}
__device__ __forceinline__ bool open_face(const StepView& s, P3 pos, int axis) {  // :32
    const P3 q = wrap_cell(s, pos);
    if (!valid_face(s, q, axis)) return false;
    P3 left = q;
    left.v[axis] -= 1;
    return fluid(s, left) && fluid(s, q);
}
__device__ __forceinline__ uint32_t face_index(const StepView& s, P3 q, int axis) {
    const uint32_t nx = s.dims[0], ny = s.dims[1];
    if (axis == 0) return (uint32_t)q.v[0] + (nx + 1) * ((uint32_t)q.v[1] + ny * (uint32_t)q.v[2]);
    if (axis == 1) return (uint32_t)q.v[0] + nx * ((uint32_t)q.v[1] + (ny + 1) * (uint32_t)q.v[2]);
    return (uint32_t)q.v[0] + nx * ((uint32_t)q.v[1] + ny * (uint32_t)q.v[2]);
}
// face() (:33-36) over the face arrays in s.vel
__device__ __forceinline__ float face(const StepView& s, P3 pos, int axis) {
    const P3 q = wrap_cell(s, pos);
    if (!open_face(s, q, axis)) return 0.0f;
    return s.vel[axis][face_index(s, q, axis)];
}
// face() over an array that already holds face() of every SoA position
// (closed faces zero, periodic positions canonical): only the wrap and the
// domain test remain.
__device__ __forceinline__ float face_masked(const StepView& s, const float* __restrict__ arr, P3 c, int axis) {
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int n = (int)s.dims[a];
        if (s.periodic & (1u << a)) {
            if (c.v[a] < 0 || c.v[a] >= n) c.v[a] = wrap_periodic(c.v[a], (uint32_t)n);
        } else if (c.v[a] < 0 || c.v[a] >= n + (a == axis ? 1 : 0)) {
            return 0.0f;
        }
    }
    return __ldg(arr + face_index(s, c, axis));
}
// open_face() from the flags ks_open_faces wrote, with face_masked's wrap
// and domain test.
__device__ __forceinline__ bool open_masked(const StepView& s, const uint8_t* __restrict__ open, P3 c, int axis) {
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int n = (int)s.dims[a];
        if (s.periodic & (1u << a)) {
            if (c.v[a] < 0 || c.v[a] >= n) c.v[a] = wrap_periodic(c.v[a], (uint32_t)n);
        } else if (c.v[a] < 0 || c.v[a] >= n + (a == axis ? 1 : 0)) {
            return false;
        }
    }
    return __ldg(open + face_index(s, c, axis)) != 0;
}
__device__ __forceinline__ float occupancy(const StepView& s, P3 pos) {
    const P3 q = wrap_cell(s, pos);
    if (!valid_cell(s, q) || !s.occ) return 0.0f;
    return s.occ[cell_index(s, q)];
}
__device__ __forceinline__ float density(const StepView& s, P3 pos) {  // :41, mix(air, liquid, alpha)
    const float t = occupancy(s, pos);
    return s.rho_air * (1.0f - t) + s.rho_l * t;
}
__device__ __forceinline__ float face_density(const StepView& s, P3 pos, int axis) {  // :42
    P3 left = pos;
    left.v[axis] -= 1;
    return 0.5f * (density(s, left) + density(s, pos));
}
__device__ __forceinline__ float mobility(const StepView& s, P3 pos, int axis) {  // :43-51
    float beta = 1.0f;
    P3 left = pos;
    left.v[axis] -= 1;
    if (s.two_phase) beta = s.rho_l / face_density(s, pos, axis);
    if (!s.phase) return beta;
    if (!fluid(s, pos) || !fluid(s, left)) return 0.0f;
    const float fa = s.phase[cell_index(s, wrap_cell(s, pos))];
    const float fb = s.phase[cell_index(s, wrap_cell(s, left))];
    const float f = fminf(fa, fb);
    const float drag = s.drag_rate * (1.0f - f) * (1.0f - f) / (f * f * f + 1e-3f);
    return beta / (1.0f + s.dt * drag);
}
__device__ __forceinline__ float em_force(const StepView& s, P3 pos, int axis) {  // :108
    const P3 q = wrap_cell(s, pos);
    if (!s.em || !valid_cell(s, q)) return 0.0f;
    const float4 f = s.em[cell_index(s, q)];
    return axis == 0 ? f.x : (axis == 1 ? f.y : f.z);
}
// The sampled grid of sample_component: extents, periodic bits and the face
// array of one component, passed by value so the sampler keeps them in
// registers.
struct SampleGrid {
    int nx, ny, nz;
    uint32_t periodic;
    const float* __restrict__ arr;
};

template <int C>
__device__ __forceinline__ float tap(const SampleGrid& g, int x, int y, int z) {
    // face() over the masked array: wrap periodic axes, zero outside the grid
    const int n[3] = {g.nx, g.ny, g.nz};
    int c[3] = {x, y, z};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        if (g.periodic & (1u << a)) {
            if (c[a] < 0 || c[a] >= n[a]) c[a] = wrap_periodic(c[a], (uint32_t)n[a]);
        } else if (c[a] < 0 || c[a] >= n[a] + (a == C ? 1 : 0)) {
            return 0.0f;
        }
    }
    const uint32_t row = (uint32_t)g.nx + (C == 0 ? 1u : 0u);
    const uint32_t col = (uint32_t)g.ny + (C == 1 ? 1u : 0u);
    return __ldg(g.arr + (uint32_t)c[0] + row * ((uint32_t)c[1] + col * (uint32_t)c[2]));
}

// The eight taps of a sample that touches the grid's edge or wraps.
template <int C>
__device__ __noinline__ float sample_edge(SampleGrid g, int bx, int by, int bz, float fx, float fy, float fz) {
    float value = 0.0f;
#pragma unroll 1
    for (int k = 0; k < 8; k++) {
        const int x = k & 1, y = (k >> 1) & 1, z = k >> 2;
        const float wx = x ? fx : 1.0f - fx;
        const float wy = y ? fy : 1.0f - fy;
        const float wz = z ? fz : 1.0f - fz;
        value += tap<C>(g, bx + x, by + y, bz + z) * wx * wy * wz;
    }
    return value;
}

// sample_component (:109-116): trilinear in the face grid of component C at
// (px, py, pz).  When all eight taps lie inside the grid without a periodic
// wrap they are read at fixed strides from one index; either way the products
// and sums are the same operations in the same order.  One out-of-line copy
// per component: inlined, unrolled samplers overflow the instruction cache.
template <int C>
__device__ __noinline__ float sample_component(SampleGrid g, float px, float py, float pz) {
    const float pos[3] = {px, py, pz};
    int base[3];
    float fraction[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float q = pos[a] - (a == C ? 0.0f : 0.5f);
        const float fl = floorf(q);
        base[a] = (int)fl;
        fraction[a] = q - fl;  // fract()
    }
    const int n[3] = {g.nx, g.ny, g.nz};
    bool inside = true;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int hi = (g.periodic & (1u << a)) ? n[a] : n[a] + (a == C ? 1 : 0);
        inside = inside && base[a] >= 0 && base[a] + 1 < hi;
    }
    float value = 0.0f;
    if (inside) {
        const uint32_t row = (uint32_t)g.nx + (C == 0 ? 1u : 0u);
        const uint32_t plane = row * ((uint32_t)g.ny + (C == 1 ? 1u : 0u));
        const float* __restrict__ p0 = g.arr + (uint32_t)base[0] + row * (uint32_t)base[1] + plane * (uint32_t)base[2];
#pragma unroll
        for (int z = 0; z < 2; z++)
#pragma unroll
            for (int y = 0; y < 2; y++)
#pragma unroll
                for (int x = 0; x < 2; x++) {
                    const float wx = x ? fraction[0] : 1.0f - fraction[0];
                    const float wy = y ? fraction[1] : 1.0f - fraction[1];
                    const float wz = z ? fraction[2] : 1.0f - fraction[2];
                    value += __ldg(p0 + (uint32_t)x + (uint32_t)y * row + (uint32_t)z * plane) * wx * wy * wz;
                }
        return value;
    }
    return sample_edge<C>(g, base[0], base[1], base[2], fraction[0], fraction[1], fraction[2]);
}

__device__ __forceinline__ bool face_position(const StepView& s, int axis, uint32_t f, P3* pos) {
    uint32_t d[3] = {s.dims[0], s.dims[1], s.dims[2]};
    d[axis] += 1;
    if (f >= d[0] * d[1] * d[2]) return false;
    pos->v[0] = (int)(f % d[0]);
    pos->v[1] = (int)((f / d[0]) % d[1]);
    pos->v[2] = (int)(f / (d[0] * d[1]));
    return true;
}

// face() and open_face() of every SoA position of one axis: the sampling
// arrays of predict and the open flags of viscous.
__global__ void ks_open_faces(StepView s, int axis, float* __restrict__ out, uint8_t* __restrict__ open) {
    const uint32_t f = blockIdx.x * WG + threadIdx.x;
    P3 pos;
    if (!face_position(s, axis, f, &pos)) return;
    out[f] = face(s, pos, axis);
    open[f] = open_face(s, pos, axis) ? 1 : 0;
}

template <int AXIS>
__global__ void ks_predict(StepView s, const float* __restrict__ m0, const float* __restrict__ m1,
                           const float* __restrict__ m2, float* __restrict__ out) {
    const uint32_t f = blockIdx.x * WG + threadIdx.x;
    P3 pos;
    if (!face_position(s, AXIS, f, &pos)) return;
    const float* m[3] = {m0, m1, m2};
    float value = 0.0f;
    if (open_face(s, pos, AXIS)) {
        const float center = face_masked(s, m[AXIS], pos, AXIS);
        value = center;
        if (s.advection) {
            const int nx = (int)s.dims[0], ny = (int)s.dims[1], nz = (int)s.dims[2];
            const SampleGrid g0{nx, ny, nz, s.periodic, m0}, g1{nx, ny, nz, s.periodic, m1},
                g2{nx, ny, nz, s.periodic, m2};
            float at[3];
            for (int a = 0; a < 3; a++) at[a] = (float)pos.v[a] + 0.5f;
            at[AXIS] -= 0.5f;
            const float v0 = sample_component<0>(g0, at[0], at[1], at[2]);
            const float v1 = sample_component<1>(g1, at[0], at[1], at[2]);
            const float v2 = sample_component<2>(g2, at[0], at[1], at[2]);
            const float half = 0.5f * s.dt / s.h;
            const float mx = at[0] - v0 * half, my = at[1] - v1 * half, mz = at[2] - v2 * half;
            const float w0 = sample_component<0>(g0, mx, my, mz);
            const float w1 = sample_component<1>(g1, mx, my, mz);
            const float w2 = sample_component<2>(g2, mx, my, mz);
            const float full = s.dt / s.h;
            const float bx = at[0] - w0 * full, by = at[1] - w1 * full, bz = at[2] - w2 * full;
            if (AXIS == 0) value = sample_component<0>(g0, bx, by, bz);
            else if (AXIS == 1) value = sample_component<1>(g1, bx, by, bz);
            else value = sample_component<2>(g2, bx, by, bz);
        }
    }
    out[f] = value;
}

// capillary_force (:52-57): sigma k (alpha_R - alpha_L) / h with the
// interface-weighted curvature of the two cells.
__device__ float capillary_force(const StepView& s, P3 pos, int axis) {
    if (!s.two_phase || !open_face(s, pos, axis)) return 0.0f;
    P3 left = pos;
    left.v[axis] -= 1;
    const float al = occupancy(s, left), ar = occupancy(s, pos);
    const float kl = s.curv ? s.curv[cell_index(s, wrap_cell(s, left))] : 0.0f;
    const float kr = s.curv ? s.curv[cell_index(s, wrap_cell(s, pos))] : 0.0f;
    const float wl = al * (1.0f - al), wr = ar * (1.0f - ar);
    const float k = wl + wr > 1e-6f ? (wl * kl + wr * kr) / fmaxf(wl + wr, 1e-20f) : 0.5f * (kl + kr);
    return s.sigma * k * (ar - al) / s.h;
}

__global__ void ks_viscous(StepView s, int axis, float* __restrict__ out) {
    const uint32_t f = blockIdx.x * WG + threadIdx.x;
    P3 pos;
    if (!face_position(s, axis, f, &pos)) return;
    const uint8_t* __restrict__ open = s.open[axis];
    float value = 0.0f;
    if (open[f]) {  // open_face(pos, axis)
        // the predicted arrays hold face() of every position (predict writes
        // zero on closed faces and the canonical value on periodic ones)
        const float* __restrict__ vel = s.vel[axis];
        bool interior = true;  // all six neighbours in the array without a wrap
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const int hi = (s.periodic & (1u << a)) ? (int)s.dims[a] : (int)s.dims[a] + (a == axis ? 1 : 0);
            interior = interior && pos.v[a] >= 1 && pos.v[a] + 1 < hi;
        }
        const float center = interior ? __ldg(vel + f) : face_masked(s, vel, pos, axis);
        float laplace = 0.0f;
        if (!s.two_phase) {
            if (interior) {
                const uint32_t row = s.dims[0] + (axis == 0 ? 1u : 0u);
                const uint32_t step[3] = {1u, row, row * (s.dims[1] + (axis == 1 ? 1u : 0u))};
#pragma unroll
                for (int d = 0; d < 3; d++)
#pragma unroll
                    for (int sign = -1; sign <= 1; sign += 2) {
                        const uint32_t q = sign < 0 ? f - step[d] : f + step[d];
                        float neighbor = __ldg(vel + q);
                        if (!__ldg(open + q) && d != axis) neighbor = -center;
                        laplace += neighbor - center;
                    }
            } else {
#pragma unroll
                for (int d = 0; d < 3; d++)
#pragma unroll
                    for (int sign = -1; sign <= 1; sign += 2) {
                        P3 q = pos;
                        q.v[d] += sign;
                        float neighbor = face_masked(s, vel, q, axis);
                        if (!open_masked(s, open, q, axis) && d != axis) neighbor = -center;
                        laplace += neighbor - center;
                    }
            }
        }
        P3 left = pos;
        left.v[axis] -= 1;
        float rho = s.rho_l, capillary = 0.0f;
        if (s.two_phase) {
            rho = face_density(s, pos, axis);
            capillary = capillary_force(s, pos, axis) / rho;
        }
        const float acc =
            s.acc[axis] + (em_force(s, left, axis) + em_force(s, pos, axis)) / (2.0f * rho) + capillary;
        float beta = mobility(s, pos, axis);
        if (s.two_phase) beta *= rho / s.rho_l;
        value = (center + s.nu * s.dt / (s.h * s.h) * laplace + s.dt * acc) * beta;
    }
    out[f] = value;
}

// ------------------------------------------------ moving-interface stresses
// src/fluid/viscosity.wgsl: symmetric Newtonian stresses on the MAC grid,
// normal stresses at cells, shear stresses at edges.
__device__ __forceinline__ P3 shifted(P3 q, int a, int d) {
    q.v[a] += d;
    return q;
}
__device__ __forceinline__ float dynamic_mu(const StepView& s, P3 q) {  // :3-6
    if (!fluid(s, q)) return 0.0f;
    const float t = fminf(fmaxf(occupancy(s, q), 0.0f), 1.0f);
    const float mu_l = s.nu * s.rho_l;
    return s.mu_air * (1.0f - t) + mu_l * t;
}
__device__ __forceinline__ float coefficient_mu(const StepView& s, P3 q, bool cached) {  // :12-16
    if (!cached) return dynamic_mu(s, q);
    const P3 at = wrap_cell(s, q);
    if (!valid_cell(s, at)) return 0.0f;
    return s.mu_c[cell_index(s, at)];
}
__device__ __forceinline__ float edge_mu(const StepView& s, P3 q, int i, int j, bool cached) {  // :17-24
    float total = 0.0f, count = 0.0f;
    for (int a = 0; a < 2; a++)
        for (int b = 0; b < 2; b++) {
            P3 at = q;
            at.v[i] -= a;
            at.v[j] -= b;
            if (fluid(s, at)) {
                total += coefficient_mu(s, at, cached);
                count += 1.0f;
            }
        }
    return total / fmaxf(count, 1.0f);
}
__device__ __forceinline__ float normal_stress(const StepView& s, P3 q, int i, bool cached) {  // :30-33
    if (!fluid(s, q)) return 0.0f;
    return 2.0f * coefficient_mu(s, q, cached) * (face(s, shifted(q, i, 1), i) - face(s, q, i)) / s.h;
}
__device__ __forceinline__ float shear_stress(const StepView& s, P3 q, int i, int j, bool cached) {  // :34-44
    const P3 lower_i = shifted(q, j, -1), lower_j = shifted(q, i, -1);
    float ui1 = face(s, q, i), ui0 = face(s, lower_i, i);
    float uj1 = face(s, q, j), uj0 = face(s, lower_j, j);
    // odd tangential ghosts: zero velocity on the wall
    if (!open_face(s, q, i) && open_face(s, lower_i, i)) ui1 = -ui0;
    if (!open_face(s, lower_i, i) && open_face(s, q, i)) ui0 = -ui1;
    if (!open_face(s, q, j) && open_face(s, lower_j, j)) uj1 = -uj0;
    if (!open_face(s, lower_j, j) && open_face(s, q, j)) uj0 = -uj1;
    return edge_mu(s, q, i, j, cached) * (ui1 - ui0 + uj1 - uj0) / s.h;
}
__device__ __forceinline__ float tensor_normal(const StepView& s, P3 q, int i) {  // :55-58
    const P3 at = wrap_cell(s, q);
    if (!valid_cell(s, at)) return 0.0f;
    const float4 t = s.t4[cell_index(s, at)];
    return i == 0 ? t.x : (i == 1 ? t.y : t.z);
}
__device__ __forceinline__ float tensor_shear(const StepView& s, P3 q, int i, int j) {  // :59-66
    const P3 at = wrap_cell(s, q);
    if (!valid_cell(s, at)) return shear_stress(s, q, i, j, true);
    const uint32_t c = cell_index(s, at);
    const int plane = i + j;
    if (plane == 1) return s.t4[c].w;
    const float2 t = s.t2[c];
    return plane == 2 ? t.x : t.y;
}
__device__ __forceinline__ float stress_acceleration(const StepView& s, P3 q, int i, bool cached) {  // :67-80
    const P3 left = shifted(q, i, -1);
    float divergence = 0.0f;
    if (cached) {
        divergence = tensor_normal(s, q, i) - tensor_normal(s, left, i);
#pragma unroll
        for (int j = 0; j < 3; j++)
            if (j != i) divergence += tensor_shear(s, shifted(q, j, 1), i, j) - tensor_shear(s, q, i, j);
    } else {
        divergence = normal_stress(s, q, i, false) - normal_stress(s, left, i, false);
#pragma unroll
        for (int j = 0; j < 3; j++)
            if (j != i)
                divergence += shear_stress(s, shifted(q, j, 1), i, j, false) - shear_stress(s, q, i, j, false);
    }
    return divergence / (s.h * face_density(s, q, i));
}
__device__ __forceinline__ P3 cell_position(const StepView& s, uint32_t i) {
    P3 q;
    q.v[0] = (int)(i % s.dims[0]);
    q.v[1] = (int)((i / s.dims[0]) % s.dims[1]);
    q.v[2] = (int)(i / (s.dims[0] * s.dims[1]));
    return q;
}

__global__ void ks_stress_coefficients(StepView s) {  // stress_coefficients (:25-29)
    const uint32_t i = blockIdx.x * WG + threadIdx.x;
    if (i >= s.dims[3]) return;
    s.mu_c[i] = dynamic_mu(s, cell_position(s, i));
}
__global__ void ks_stress_tensor(StepView s) {  // stress_tensor (:47-54)
    const uint32_t i = blockIdx.x * WG + threadIdx.x;
    if (i >= s.dims[3]) return;
    const P3 q = cell_position(s, i);
    s.t4[i] = make_float4(normal_stress(s, q, 0, true), normal_stress(s, q, 1, true), normal_stress(s, q, 2, true),
                          shear_stress(s, q, 0, 1, true));
    s.t2[i] = make_float2(shear_stress(s, q, 0, 2, true), shear_stress(s, q, 1, 2, true));
}
__global__ void ks_stress_save_initial(StepView s) {  // stress_save_initial (stabilized.wgsl:6-15)
    const uint32_t i = blockIdx.x * WG + threadIdx.x;
    if (i >= s.dims[3]) return;
    const P3 q = cell_position(s, i);
    float y[3] = {0.0f, 0.0f, 0.0f}, op[3] = {0.0f, 0.0f, 0.0f};
    for (int axis = 0; axis < 3; axis++)
        if (open_face(s, q, axis)) {
            y[axis] = face(s, q, axis);
            op[axis] = stress_acceleration(s, q, axis, true);
        }
    s.y0[i] = make_float4(y[0], y[1], y[2], 0.0f);
    s.f0[i] = make_float4(op[0], op[1], op[2], 0.0f);
}
// stress_stabilized (stabilized.wgsl:16-30): io holds the stage before the
// previous one (read) and receives the new stage; s.vel the previous stage.
template <int AXIS>
__global__ void ks_stress_stage(StepView s, float bx, float by, float bz, float bw, float ix, float* __restrict__ io) {
    constexpr int axis = AXIS;
    const uint32_t f = blockIdx.x * WG + threadIdx.x;
    P3 pos;
    if (!face_position(s, axis, f, &pos)) return;
    const float older = io[f];
    float value = 0.0f;
    if (open_face(s, pos, axis)) {
        const uint32_t cell = cell_index(s, wrap_cell(s, pos));
        const float previous = face(s, pos, axis);
        const float4 y = s.y0[cell], op = s.f0[cell];
        const float initial = axis == 0 ? y.x : (axis == 1 ? y.y : y.z);
        const float initial_op = axis == 0 ? op.x : (axis == 1 ? op.y : op.z);
        value = bx * previous + by * older + bz * initial + bw * stress_acceleration(s, pos, axis, true) +
                ix * initial_op;
    }
    io[f] = value;
}
// The uncached stress operator of stress_diffuse evaluated from per-cell
// stresses: the 3 normal stresses and the shear stress of every ordered axis
// pair (i, j) (the operator evaluates shear(q, i, j) for the face axis i, so
// both orders are kept: they sum in different orders).  The cached cell
// viscosity equals dynamic_mu() wherever the uncached operator reads it, so
// every stress, and so every result, is the one the uncached operator
// computes.  Layout: 9 planes of n floats.
__device__ __forceinline__ int pair_slot(int i, int j) { return 3 + 2 * i + (j > i ? j - 1 : j); }
// Interior cells (every neighbour the stresses touch inside the grid, no
// wrap): the same stresses from ten fluid flags, seven cell viscosities and
// twelve face values read at fixed strides.  F/M/U below follow face(),
// open_face(), coefficient_mu() and edge_mu() term by term.
__device__ __forceinline__ void stress_cells_interior(const StepView& s, uint32_t i, P3 q, float* __restrict__ t9) {
    const uint32_t nx = s.dims[0], ny = s.dims[1];
    const size_t n = s.dims[3];
    const uint32_t cs[3] = {1u, nx, nx * ny};
    // face index of position q in each axis array, and the strides of that array
    const uint32_t fi[3] = {(uint32_t)q.v[0] + (nx + 1) * ((uint32_t)q.v[1] + ny * (uint32_t)q.v[2]),
                            (uint32_t)q.v[0] + nx * ((uint32_t)q.v[1] + (ny + 1) * (uint32_t)q.v[2]), i};
    const uint32_t fs[3][3] = {{1u, nx + 1, (nx + 1) * ny}, {1u, nx, nx * (ny + 1)}, {1u, nx, nx * ny}};
    auto F = [&](int dx, int dy, int dz) {
        return is_fluid_index(s, i + (uint32_t)(dx * (int)cs[0] + dy * (int)cs[1] + dz * (int)cs[2]));
    };
    auto M = [&](int dx, int dy, int dz) {
        return s.mu_c[i + (uint32_t)(dx * (int)cs[0] + dy * (int)cs[1] + dz * (int)cs[2])];
    };
    const bool f0 = F(0, 0, 0);
    const bool fm[3] = {F(-1, 0, 0), F(0, -1, 0), F(0, 0, -1)};
    const bool fp[3] = {F(1, 0, 0), F(0, 1, 0), F(0, 0, 1)};
    // fluid(q - e_a - e_b), a < b: (0,1), (0,2), (1,2)
    const bool fmm[3] = {F(-1, -1, 0), F(-1, 0, -1), F(0, -1, -1)};
    auto fmm_of = [&](int a, int b) { return fmm[a + b - 1]; };
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float v = 0.0f;
        if (f0) {
            const float lo = (fm[a] && f0) ? __ldg(s.vel[a] + fi[a]) : 0.0f;
            const float hi = (f0 && fp[a]) ? __ldg(s.vel[a] + fi[a] + fs[a][a]) : 0.0f;
            v = 2.0f * s.mu_c[i] * (hi - lo) / s.h;
        }
        t9[a * n + i] = v;
    }
    const float mu0 = s.mu_c[i];
    const float mum[3] = {M(-1, 0, 0), M(0, -1, 0), M(0, 0, -1)};
    const float mumm[3] = {M(-1, -1, 0), M(-1, 0, -1), M(0, -1, -1)};
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) {
            if (a == b) continue;
            // faces: (q, a), (q - e_b, a), (q, b), (q - e_a, b)
            const bool o_ai1 = fm[a] && f0;               // open_face(q, a)
            const bool o_ai0 = fmm_of(a, b) && fm[b];     // open_face(q - e_b, a)
            const bool o_bj1 = fm[b] && f0;               // open_face(q, b)
            const bool o_bj0 = fmm_of(a, b) && fm[a];     // open_face(q - e_a, b)
            float ui1 = o_ai1 ? __ldg(s.vel[a] + fi[a]) : 0.0f;
            float ui0 = o_ai0 ? __ldg(s.vel[a] + fi[a] - fs[a][b]) : 0.0f;
            float uj1 = o_bj1 ? __ldg(s.vel[b] + fi[b]) : 0.0f;
            float uj0 = o_bj0 ? __ldg(s.vel[b] + fi[b] - fs[b][a]) : 0.0f;
            if (!o_ai1 && o_ai0) ui1 = -ui0;
            if (!o_ai0 && o_ai1) ui0 = -ui1;
            if (!o_bj1 && o_bj0) uj1 = -uj0;
            if (!o_bj0 && o_bj1) uj0 = -uj1;
            // edge_mu(q, a, b): cells q, q - e_b, q - e_a, q - e_a - e_b in that order
            float total = 0.0f, count = 0.0f;
            if (f0) { total += mu0; count += 1.0f; }
            if (fm[b]) { total += mum[b]; count += 1.0f; }
            if (fm[a]) { total += mum[a]; count += 1.0f; }
            if (fmm_of(a, b)) { total += mumm[a + b - 1]; count += 1.0f; }
            const float emu = total / fmaxf(count, 1.0f);
            t9[pair_slot(a, b) * n + i] = emu * (ui1 - ui0 + uj1 - uj0) / s.h;
        }
}
__device__ __forceinline__ bool stress_interior(const StepView& s, P3 q) {
    bool interior = true;
#pragma unroll
    for (int a = 0; a < 3; a++) interior = interior && q.v[a] >= 1 && q.v[a] + 2 <= (int)s.dims[a];
    return interior;
}
// Two launches over the cells, interior cells in one and the cells on the
// grid's faces (the general stresses) in the other, so that no warp runs both
// paths and each kernel's code stays small.
__global__ void ks_stress_cells(StepView s, float* __restrict__ t9) {
    const uint32_t i = blockIdx.x * WG + threadIdx.x;
    if (i >= s.dims[3]) return;
    const P3 q = cell_position(s, i);
    if (stress_interior(s, q)) stress_cells_interior(s, i, q, t9);
}
// The shell of a box of extents d (positions with a coordinate at 0 or
// d - 1), numbered densely so consecutive lanes take consecutive positions:
// the z = 0 and z = d2-1 planes, the y = 0 and y = d1-1 rows of the planes
// between, then the x = 0 and x = d0-1 positions of the rows between.  A box
// with an extent below 3 has no interior: every position is listed.
__host__ __device__ inline uint64_t shell_count(const int d[3]) {
    const uint64_t n = (uint64_t)d[0] * d[1] * d[2];
    if (d[0] < 3 || d[1] < 3 || d[2] < 3) return n;
    return n - (uint64_t)(d[0] - 2) * (d[1] - 2) * (d[2] - 2);
}
__device__ __forceinline__ bool shell_position(const int d[3], uint32_t t, P3* q) {
    const int nx = d[0], ny = d[1], nz = d[2];
    if (nx < 3 || ny < 3 || nz < 3) {
        if ((uint64_t)t >= (uint64_t)nx * ny * nz) return false;
        q->v[0] = (int)(t % nx);
        q->v[1] = (int)((t / nx) % ny);
        q->v[2] = (int)(t / ((uint32_t)nx * ny));
        return true;
    }
    const uint32_t plane = (uint32_t)(nx * ny), rows = (uint32_t)(2 * nx * (nz - 2)), cols = (uint32_t)(2 * (ny - 2) * (nz - 2));
    if (t < 2 * plane) {
        const uint32_t r = t % plane;
        q->v[0] = (int)(r % nx);
        q->v[1] = (int)(r / nx);
        q->v[2] = t < plane ? 0 : nz - 1;
        return true;
    }
    t -= 2 * plane;
    if (t < rows) {
        const uint32_t half = (uint32_t)(nx * (nz - 2)), r = t % half;
        q->v[0] = (int)(r % nx);
        q->v[1] = t < half ? 0 : ny - 1;
        q->v[2] = 1 + (int)(r / nx);
        return true;
    }
    t -= rows;
    if (t < cols) {
        const uint32_t half = (uint32_t)((ny - 2) * (nz - 2)), r = t % half;
        q->v[0] = t < half ? 0 : nx - 1;
        q->v[1] = 1 + (int)(r % (ny - 2));
        q->v[2] = 1 + (int)(r / (ny - 2));
        return true;
    }
    return false;
}
__host__ __device__ inline void cell_extents(const StepView& s, int d[3]) {
    d[0] = (int)s.dims[0];
    d[1] = (int)s.dims[1];
    d[2] = (int)s.dims[2];
}
__global__ void ks_stress_cells_edge(StepView s, float* __restrict__ t9) {
    P3 q;
    int d[3];
    cell_extents(s, d);
    if (!shell_position(d, blockIdx.x * WG + threadIdx.x, &q)) return;
    const uint32_t i = cell_index(s, q);
    const size_t n = s.dims[3];
    // compact loops: this kernel runs few cells, and unrolled general stresses
    // overflow the instruction cache
#pragma unroll 1
    for (int a = 0; a < 3; a++) t9[a * n + i] = normal_stress(s, q, a, true);
#pragma unroll 1
    for (int a = 0; a < 3; a++)
#pragma unroll 1
        for (int b = 0; b < 3; b++)
            if (a != b) t9[pair_slot(a, b) * n + i] = shear_stress(s, q, a, b, true);
}
__device__ __forceinline__ float cell_normal(const StepView& s, const float* __restrict__ t9, P3 q, int i) {
    const P3 at = wrap_cell(s, q);
    if (!valid_cell(s, at)) return 0.0f;  // normal_stress: not a fluid cell
    return t9[(size_t)i * s.dims[3] + cell_index(s, at)];
}
// Shear stresses one layer past the high faces of the grid (q[j] = n_j; the
// Euler operator reads shear(pos + e_j, i, j) there): for each j the plane of
// the other two axes a < b, for i = a then i = b.  Layout: j = 0 planes, then
// j = 1, then j = 2.
__device__ __forceinline__ size_t ghost_index(const StepView& s, P3 q, int i, int j) {
    const int a = j == 0 ? 1 : 0, b = j == 2 ? 1 : 2;
    const size_t plane = (size_t)s.dims[a] * s.dims[b];
    size_t base = 0;
    if (j >= 1) base += 2ull * s.dims[1] * s.dims[2];
    if (j >= 2) base += 2ull * s.dims[0] * s.dims[2];
    return base + (i == a ? 0 : plane) + (size_t)q.v[a] + (size_t)s.dims[a] * (size_t)q.v[b];
}
__host__ __device__ inline uint64_t ghost_count(const StepView& s) {
    return 2ull * ((uint64_t)s.dims[1] * s.dims[2] + (uint64_t)s.dims[0] * s.dims[2] + (uint64_t)s.dims[0] * s.dims[1]);
}
__global__ void ks_stress_ghosts(StepView s, float* __restrict__ g) {
    uint64_t t = (uint64_t)blockIdx.x * WG + threadIdx.x;
    if (t >= ghost_count(s)) return;
    int j = 0;
    for (; j < 3; j++) {
        const int a = j == 0 ? 1 : 0, b = j == 2 ? 1 : 2;
        const uint64_t span = 2ull * s.dims[a] * s.dims[b];
        if (t < span) break;
        t -= span;
    }
    const int a = j == 0 ? 1 : 0, b = j == 2 ? 1 : 2;
    const uint64_t plane = (uint64_t)s.dims[a] * s.dims[b];
    const int i = t < plane ? a : b;
    const uint64_t r = t % plane;
    P3 q;
    q.v[j] = (int)s.dims[j];
    q.v[a] = (int)(r % s.dims[a]);
    q.v[b] = (int)(r / s.dims[a]);
    g[ghost_index(s, q, i, j)] = shear_stress(s, q, i, j, true);
}
__device__ __forceinline__ float cell_shear(const StepView& s, const float* __restrict__ t9, P3 q, int i, int j) {
    const P3 at = wrap_cell(s, q);
    if (!valid_cell(s, at)) return t9[9ull * s.dims[3] + ghost_index(s, q, i, j)];  // one past a high face
    return t9[(size_t)pair_slot(i, j) * s.dims[3] + cell_index(s, at)];
}
// stress_diffuse (:100-107): one explicit Euler substep.
template <int AXIS>
__global__ void ks_stress_diffuse(StepView s, float dt_sub, const float* __restrict__ t9, float* __restrict__ out) {
    constexpr int axis = AXIS;
    const uint32_t f = blockIdx.x * WG + threadIdx.x;
    P3 pos;
    if (!face_position(s, axis, f, &pos)) return;
    float value = 0.0f;
    if (open_face(s, pos, axis)) {
        const P3 left = shifted(pos, axis, -1);
        float divergence = cell_normal(s, t9, pos, axis) - cell_normal(s, t9, left, axis);
#pragma unroll
        for (int j = 0; j < 3; j++)
            if (j != axis)
                divergence += cell_shear(s, t9, shifted(pos, j, 1), axis, j) - cell_shear(s, t9, pos, axis, j);
        const float acc = divergence / (s.h * face_density(s, pos, axis));
        value = face(s, pos, axis) + dt_sub * acc;
    }
    out[f] = value;
}
// viscosity_bound (:81-96): 4 x the absolute row sum of rho^-1 div(tau) over
// the open faces; the block maximum goes to *bound_bits as float bits (all
// values are non-negative, so the unsigned maximum is the float maximum).
// The bound of an interior face (every cell it reads inside the grid, no
// wrap): cell viscosities and fluid flags by fixed strides, summed in the
// order of the general expression below.
template <int AXIS>
__device__ __forceinline__ float viscosity_bound_interior(const StepView& s, P3 q, bool* open) {
    const uint32_t nx = s.dims[0], ny = s.dims[1];
    const int cs[3] = {1, (int)nx, (int)(nx * ny)};
    const uint32_t c = cell_index(s, q), l = c - (uint32_t)cs[AXIS];
    *open = is_fluid_index(s, l) && is_fluid_index(s, c);
    if (!*open) return 0.0f;
    float sum = s.mu_c[c] + s.mu_c[l];
#pragma unroll
    for (int j = 0; j < 3; j++) {
        if (j == AXIS) continue;
        const uint32_t d = (uint32_t)cs[j];
        // edge_mu(q, AXIS, j): q, q - e_j, q - e_AXIS, q - e_AXIS - e_j
        float t1 = 0.0f, n1 = 0.0f;
        const uint32_t e1[4] = {c, c - d, l, l - d};
#pragma unroll
        for (int k = 0; k < 4; k++)
            if (is_fluid_index(s, e1[k])) {
                t1 += s.mu_c[e1[k]];
                n1 += 1.0f;
            }
        // edge_mu(q + e_j, AXIS, j): q + e_j, q, q + e_j - e_AXIS, q - e_AXIS
        float t2 = 0.0f, n2 = 0.0f;
        const uint32_t e2[4] = {c + d, c, l + d, l};
#pragma unroll
        for (int k = 0; k < 4; k++)
            if (is_fluid_index(s, e2[k])) {
                t2 += s.mu_c[e2[k]];
                n2 += 1.0f;
            }
        sum += t1 / fmaxf(n1, 1.0f) + t2 / fmaxf(n2, 1.0f);
    }
    const float al = s.occ[l], ar = s.occ[c];
    const float rl = s.rho_air * (1.0f - al) + s.rho_l * al, rr = s.rho_air * (1.0f - ar) + s.rho_l * ar;
    return 4.0f * sum / (0.5f * (rl + rr) * s.h * s.h);
}
__device__ __forceinline__ void block_max_to(float bound, unsigned int* bound_bits) {
    __shared__ float red[WG];
    red[threadIdx.x] = bound;
    __syncthreads();
    for (int d = WG / 2; d > 0; d /= 2) {
        if ((int)threadIdx.x < d) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + d]);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const float b = red[0];
        // a non-finite bound is kept as the largest bit pattern: the host rejects it
        atomicMax(bound_bits, (b == b) ? __float_as_uint(b) : 0xFFFFFFFFu);
    }
}
// The face grid of AXIS: extents n + 1 along AXIS.  Its interior (shell
// excluded) is exactly the faces whose cells all lie inside the grid.
template <int AXIS>
__host__ __device__ inline void face_extents(const StepView& s, int d[3]) {
    cell_extents(s, d);
    d[AXIS] += 1;
}
template <int AXIS>
__device__ __forceinline__ float viscosity_bound_general(const StepView& s, P3 q) {
    constexpr int axis = AXIS;
    if (!open_face(s, q, axis)) return 0.0f;
    const P3 left = shifted(q, axis, -1);
    // the cached cell viscosity (ks_stress_coefficients) equals dynamic_mu()
    float sum = coefficient_mu(s, q, true) + coefficient_mu(s, left, true);
#pragma unroll
    for (int j = 0; j < 3; j++)
        if (j != axis) sum += edge_mu(s, q, axis, j, true) + edge_mu(s, shifted(q, j, 1), axis, j, true);
    return 4.0f * sum / (face_density(s, q, axis) * s.h * s.h);
}
// viscosity_bound (:81-96): 4 x the absolute row sum of rho^-1 div(tau) over
// the open faces, maximum over faces into *bound_bits as float bits (values
// are non-negative, so the unsigned maximum is the float maximum).  Interior
// faces here, the face grid's shell in ks_viscosity_bound_edge.
template <int AXIS>
__global__ void ks_viscosity_bound(StepView s, unsigned int* bound_bits) {
    const uint32_t f = blockIdx.x * WG + threadIdx.x;
    float bound = 0.0f;
    P3 q;
    int d[3];
    face_extents<AXIS>(s, d);
    if (face_position(s, AXIS, f, &q)) {
        bool interior = true;
#pragma unroll
        for (int a = 0; a < 3; a++) interior = interior && q.v[a] >= 1 && q.v[a] + 2 <= d[a];
        if (interior) {
            bool open;
            bound = s.occ ? viscosity_bound_interior<AXIS>(s, q, &open) : viscosity_bound_general<AXIS>(s, q);
        }
    }
    block_max_to(bound, bound_bits);
}
template <int AXIS>
__global__ void ks_viscosity_bound_edge(StepView s, unsigned int* bound_bits) {
    P3 q;
    int d[3];
    face_extents<AXIS>(s, d);
    const float bound = shell_position(d, blockIdx.x * WG + threadIdx.x, &q) ? viscosity_bound_general<AXIS>(s, q) : 0.0f;
    block_max_to(bound, bound_bits);
}

__global__ void ks_fields(StepView s, float4* __restrict__ cells, float4* __restrict__ partials) {
    __shared__ float4 ra[WG], rb[WG];
    __shared__ float2 rc[WG];
    const int l = threadIdx.x;
    const uint32_t i = blockIdx.x * WG + l;
    const uint32_t groups = gridDim.x;
    float4 stats = make_float4(0.f, 0.f, 0.f, 0.f), other = make_float4(0.f, 0.f, 0.f, 0.f);
    float max_face = 0.0f, melt = 0.0f;
    if (i < s.dims[3]) {
        float4 o0 = make_float4(0.f, 0.f, 0.f, 0.f), o1 = o0, o2 = o0, o3 = o0;
        const float oy = s.phase ? s.phase[i] : 0.0f;
        const float oz = s.occ ? s.occ[i] : 0.0f;
        const float ow = s.curv ? s.curv[i] : 0.0f;
        if (s.two_phase) o3 = make_float4(0.0f, oy, oz, ow);
        if (is_fluid_index(s, i)) {
            P3 pos;
            pos.v[0] = (int)(i % s.dims[0]);
            pos.v[1] = (int)((i / s.dims[0]) % s.dims[1]);
            pos.v[2] = (int)(i / (s.dims[0] * s.dims[1]));
            float v[3], face_energy = 0.0f, div = 0.0f;
            // Inside the grid (no wrap, no edge) a face of this fluid cell is
            // open exactly when the neighbour across it is fluid.
            bool interior = true;
#pragma unroll
            for (int a = 0; a < 3; a++) interior = interior && pos.v[a] >= 1 && pos.v[a] + 1 < (int)s.dims[a];
            const uint32_t nx = s.dims[0], ny = s.dims[1];
            const uint32_t cstep[3] = {1u, nx, nx * ny};
            const uint32_t flo[3] = {(uint32_t)pos.v[0] + (nx + 1) * ((uint32_t)pos.v[1] + ny * (uint32_t)pos.v[2]),
                                     (uint32_t)pos.v[0] + nx * ((uint32_t)pos.v[1] + (ny + 1) * (uint32_t)pos.v[2]),
                                     i};
            const uint32_t fstep[3] = {1u, nx, nx * ny};
#pragma unroll
            for (int axis = 0; axis < 3; axis++) {
                P3 q = pos;
                q.v[axis] += 1;
                float a, b;
                if (interior) {
                    a = is_fluid_index(s, i - cstep[axis]) ? __ldg(s.vel[axis] + flo[axis]) : 0.0f;
                    b = is_fluid_index(s, i + cstep[axis]) ? __ldg(s.vel[axis] + flo[axis] + fstep[axis]) : 0.0f;
                } else {
                    a = face(s, pos, axis);
                    b = face(s, q, axis);
                }
                v[axis] = 0.5f * (a + b);
                face_energy += 0.5f * (a * a + b * b);
                max_face = fmaxf(max_face, fmaxf(fabsf(a), fabsf(b)));
                div += b - a;  // divergence(pos, false), :104-106
            }
            div = div / s.h;
            melt = s.phase ? oy : 1.0f;
            if (s.two_phase) melt *= oz;
            const float speed = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            const float x = s.phi[(size_t)i * s.phi_stride];
            const float pv = s.mean_free ? x - s.phi[(size_t)(s.mask[i] >> 2u) * s.phi_stride] : x;
            const float pressure = pv * s.rho_l / s.dt;
            float force[3];
            for (int a = 0; a < 3; a++) force[a] = s.rho_l * s.acc[a] + em_force(s, pos, a);
            o0 = make_float4(v[0], v[1], v[2], speed);
            o1 = make_float4(pressure, div, 0.0f, 0.0f);
            o2 = make_float4(force[0], force[1], force[2], 0.0f);
            o3 = make_float4(1.0f, s.phase ? oy : 1.0f, oz, ow);
            bool bad = v[0] != v[0] || v[1] != v[1] || v[2] != v[2];
            bad = bad || force[0] != force[0] || force[1] != force[1] || force[2] != force[2];
            bad = bad || fabsf(force[0]) > 1e30f || fabsf(force[1]) > 1e30f || fabsf(force[2]) > 1e30f;
            bad = bad || speed > 1e25f || !(fabsf(pressure) < 1e30f) || !(fabsf(div) < 1e30f);
            const float rho = s.two_phase ? density(s, pos) : s.rho_l;
            stats = make_float4(speed, fabsf(div), div * div, 0.5f * rho * face_energy * s.h * s.h * s.h);
            other = make_float4(fabsf(pressure), div,
                                sqrtf(force[0] * force[0] + force[1] * force[1] + force[2] * force[2]),
                                bad ? 1.0f : 0.0f);
        }
        if (cells) {
            float4* c = cells + (size_t)4 * i;
            c[0] = o0;
            c[1] = o1;
            c[2] = o2;
            c[3] = o3;
        }
    }
    ra[l] = stats;
    rb[l] = other;
    rc[l] = make_float2(max_face, melt);
    __syncthreads();
    for (int st = 128; st > 0; st /= 2) {
        if (l < st) {
            const float4 a = ra[l], a2 = ra[l + st], b = rb[l], b2 = rb[l + st];
            ra[l] = make_float4(fmaxf(a.x, a2.x), fmaxf(a.y, a2.y), a.z + a2.z, a.w + a2.w);
            rb[l] = make_float4(fmaxf(b.x, b2.x), b.y + b2.y, fmaxf(b.z, b2.z), b.w + b2.w);
            rc[l] = make_float2(fmaxf(rc[l].x, rc[l + st].x), rc[l].y + rc[l + st].y);
        }
        __syncthreads();
    }
    if (l == 0) {
        partials[blockIdx.x] = ra[0];
        partials[groups + blockIdx.x] = rb[0];
        partials[2 * groups + blockIdx.x] = make_float4(rc[0].x, rc[0].y, 0.0f, 0.0f);
    }
}

__global__ void ks_diagnostics(const float4* __restrict__ partials, uint32_t groups, float4* __restrict__ out) {
    __shared__ float4 ra[WG], rb[WG];
    __shared__ float2 rc[WG];
    const int l = threadIdx.x;
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
    float2 c = make_float2(0.f, 0.f);
    for (uint32_t i = (uint32_t)l; i < groups; i += WG) {
        const float4 fs = partials[2 * groups + i], x = partials[i], y = partials[groups + i];
        c = make_float2(fmaxf(c.x, fs.x), c.y + fs.y);
        a = make_float4(fmaxf(a.x, x.x), fmaxf(a.y, x.y), a.z + x.z, a.w + x.w);
        b = make_float4(fmaxf(b.x, y.x), b.y + y.y, fmaxf(b.z, y.z), b.w + y.w);
    }
    ra[l] = a;
    rb[l] = b;
    rc[l] = c;
    __syncthreads();
    for (int st = 128; st > 0; st /= 2) {
        if (l < st) {
            const float4 p = ra[l], p2 = ra[l + st], q = rb[l], q2 = rb[l + st];
            ra[l] = make_float4(fmaxf(p.x, p2.x), fmaxf(p.y, p2.y), p.z + p2.z, p.w + p2.w);
            rb[l] = make_float4(fmaxf(q.x, q2.x), q.y + q2.y, fmaxf(q.z, q2.z), q.w + q2.w);
            rc[l] = make_float2(fmaxf(rc[l].x, rc[l + st].x), rc[l].y + rc[l + st].y);
        }
        __syncthreads();
    }
    if (l == 0) {
        out[0] = ra[0];
        out[1] = rb[0];
        out[2] = make_float4(rc[0].x, rc[0].y, 0.0f, 0.0f);
    }
}
}  // namespace

static unsigned face_blocks(const StepView& s, int axis) {
    uint64_t d[3] = {s.dims[0], s.dims[1], s.dims[2]};
    d[axis] += 1;
    return (unsigned)((d[0] * d[1] * d[2] + WG - 1) / WG);
}

void launch_predict(const StepView& s, float* const out[3], float* const masked[3], uint8_t* const open[3],
                    cudaStream_t st) {
    for (int a = 0; a < 3; a++) ks_open_faces<<<face_blocks(s, a), WG, 0, st>>>(s, a, masked[a], open[a]);
    ks_predict<0><<<face_blocks(s, 0), WG, 0, st>>>(s, masked[0], masked[1], masked[2], out[0]);
    ks_predict<1><<<face_blocks(s, 1), WG, 0, st>>>(s, masked[0], masked[1], masked[2], out[1]);
    ks_predict<2><<<face_blocks(s, 2), WG, 0, st>>>(s, masked[0], masked[1], masked[2], out[2]);
}
void launch_viscous(const StepView& s, float* const out[3], cudaStream_t st) {
    for (int a = 0; a < 3; a++) ks_viscous<<<face_blocks(s, a), WG, 0, st>>>(s, a, out[a]);
}
static unsigned cell_blocks(const StepView& s) { return (s.dims[3] + WG - 1) / WG; }
void launch_stress_coefficients(const StepView& s, cudaStream_t st) {
    ks_stress_coefficients<<<cell_blocks(s), WG, 0, st>>>(s);
}
void launch_stress_tensor(const StepView& s, cudaStream_t st) { ks_stress_tensor<<<cell_blocks(s), WG, 0, st>>>(s); }
void launch_stress_save_initial(const StepView& s, cudaStream_t st) {
    ks_stress_save_initial<<<cell_blocks(s), WG, 0, st>>>(s);
}
void launch_stress_stage(const StepView& s, const float row[5], float* const io[3], cudaStream_t st) {
    ks_stress_stage<0><<<face_blocks(s, 0), WG, 0, st>>>(s, row[0], row[1], row[2], row[3], row[4], io[0]);
    ks_stress_stage<1><<<face_blocks(s, 1), WG, 0, st>>>(s, row[0], row[1], row[2], row[3], row[4], io[1]);
    ks_stress_stage<2><<<face_blocks(s, 2), WG, 0, st>>>(s, row[0], row[1], row[2], row[3], row[4], io[2]);
}
void launch_stress_diffuse(const StepView& s, float dt_sub, float* t9, float* const out[3], cudaStream_t st) {
    ks_stress_cells<<<cell_blocks(s), WG, 0, st>>>(s, t9);
    int d[3];
    cell_extents(s, d);
    ks_stress_cells_edge<<<(unsigned)((shell_count(d) + WG - 1) / WG), WG, 0, st>>>(s, t9);
    ks_stress_ghosts<<<(unsigned)((ghost_count(s) + WG - 1) / WG), WG, 0, st>>>(s, t9 + 9ull * s.dims[3]);
    ks_stress_diffuse<0><<<face_blocks(s, 0), WG, 0, st>>>(s, dt_sub, t9, out[0]);
    ks_stress_diffuse<1><<<face_blocks(s, 1), WG, 0, st>>>(s, dt_sub, t9, out[1]);
    ks_stress_diffuse<2><<<face_blocks(s, 2), WG, 0, st>>>(s, dt_sub, t9, out[2]);
}
template <int AXIS>
static void viscosity_bound_axis(const StepView& s, unsigned int* bound_bits, cudaStream_t st) {
    int d[3];
    face_extents<AXIS>(s, d);
    ks_viscosity_bound<AXIS><<<face_blocks(s, AXIS), WG, 0, st>>>(s, bound_bits);
    ks_viscosity_bound_edge<AXIS><<<(unsigned)((shell_count(d) + WG - 1) / WG), WG, 0, st>>>(s, bound_bits);
}
void launch_viscosity_bound(const StepView& s, unsigned int* bound_bits, cudaStream_t st) {
    viscosity_bound_axis<0>(s, bound_bits, st);
    viscosity_bound_axis<1>(s, bound_bits, st);
    viscosity_bound_axis<2>(s, bound_bits, st);
}
uint32_t fields_groups(const StepView& s) { return (s.dims[3] + WG - 1) / WG; }
void launch_fields(const StepView& s, float4* cells, float4* partials, float4* scalars3, cudaStream_t st) {
    const uint32_t groups = fields_groups(s);
    ks_fields<<<groups, WG, 0, st>>>(s, cells, partials);
    ks_diagnostics<<<1, WG, 0, st>>>(partials, groups, scalars3);
}

}  // namespace mhdproj
