/*
 * oracle_em.c -- CPU restatement of the reference's implicit EM induction
 * solve, used only by the tests and the benchmark's CPU leg to check the
 * library's GPU path.  It is not part of the product.
 *
 * Source followed:
 *   src/em/common.wgsl:1-11      grid parameters and edge indexing
 *   src/em/induction.wgsl:16-104 material coefficients, curl, adjoint,
 *                                gauge, mass and diagonal
 *   src/em/induction.wgsl:105-267 the passes (coefficients, prepare,
 *                                initial_reduce, apply_operator,
 *                                alpha_reduce, update_residual,
 *                                beta_reduce, update_search,
 *                                true_residual, restart_reduce, fields,
 *                                field_reduce, begin_step, zero_guess,
 *                                commit_step, rollback, hold_source)
 *   src/em/source.wgsl:16-17     history shift of the applied potential
 *   src/em/mod.rs:863-1090       EmState::advance_to: the host sequence
 *                                (scale repeat, prediction guard, 32-pass
 *                                batches, true-residual restarts,
 *                                acceptance, rollback, prediction history)
 *   src/em/grid.rs:13-36         the physical constants (dt, mu0, h, tol^2)
 *
 * Arithmetic is FP32 in the shader's operation order (compile with
 * -ffp-contract=off); workgroup sums are 256-lane trees and the single-group
 * reductions accumulate partials with a stride of 256 before their tree, as
 * the shader does.  Records keep the shader's vec4 layout:
 *   source[i]     = (A_s now, A_s previous, sigma_edge, diagonal)
 *   source[E + i] = (motional EMF, lower air node, upper air node, air stencil)
 *   work[i]       = (reaction increment x, r, p, A p or diagonal)
 * mix(e1, e2, t) is e1*(1-t) + e2*t and length(v) is sqrt((x*x + y*y) + z*z).
 *
 *   src/em/nodal.wgsl            the additive nodal gradient correction the
 *                                solve switches to after 1024 iterations
 *   src/em/motion.wgsl:8-26      the motional EMF
 *
 *   src/em/source.wgsl:5-17      the applied potential of source elements
 *
 *   src/em/body-stats.wgsl       per-body force and power integrals
 *   src/em/energy.wgsl           the energy ledger of a committed step
 *
 * Out of scope, as in the library: building the source elements from the
 * model (src/em/sources.rs).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "mhd_oracle.h"

typedef struct { float x, y, z, w; } f4;

struct OEm {
    uint32_t dims[4], edges[4], control[4];
    float origin[4], physical[4];
    uint32_t *materials;
    float *props;
    uint32_t n_props;
    int bad_id;
    f4 *source, *work, *partials, *results, *checkpoint;
    float *previous;
    f4 scalars[8];
    double dt_s, time_s, last_dt;
    float rel_tol;
    uint32_t max_it;
    int can_predict;
    uint32_t nodal_after; /* iterations before the nodal switch (1024 in the reference) */
    float *nodal;         /* (nx+1)(ny+1)(nz+1) nodal corrections */
    int no_predict;       /* the reference's test switch predict_increments = false */
    float prediction[3];  /* its prediction_diagnostic: factor, initial residual, fallback */
};

static f4 F4(float x, float y, float z, float w) { f4 r = {x, y, z, w}; return r; }
static f4 add4(f4 a, f4 b) { return F4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
static float maxf(float a, float b) { return a > b ? a : b; }
static float minf(float a, float b) { return a < b ? a : b; }

/* ---- grid and edge indexing (common.wgsl) ---- */
static int valid3(const int p[3], const uint32_t d[3]) {
    return p[0] >= 0 && p[1] >= 0 && p[2] >= 0 && p[0] < (int)d[0] && p[1] < (int)d[1] && p[2] < (int)d[2];
}
static void edge_dims(const OEm *s, int axis, uint32_t d[3]) {
    for (int k = 0; k < 3; k++) d[k] = s->dims[k] + 1;
    d[axis] -= 1;
}
static void face_dims(const OEm *s, int axis, uint32_t d[3]) {
    for (int k = 0; k < 3; k++) d[k] = s->dims[k];
    d[axis] += 1;
}
static uint32_t edge_offset(const OEm *s, int axis) {
    return axis == 0 ? 0 : axis == 1 ? s->edges[0] : s->edges[0] + s->edges[1];
}
static uint32_t edge_index(const OEm *s, int axis, const int p[3]) {
    uint32_t d[3];
    edge_dims(s, axis, d);
    return edge_offset(s, axis) + (uint32_t)p[0] + d[0] * ((uint32_t)p[1] + d[1] * (uint32_t)p[2]);
}
static void edge_decode(const OEm *s, uint32_t i, int p[3], int *axis) {
    int a = 0;
    uint32_t q = i;
    if (q >= s->edges[0]) {
        a = 1;
        q -= s->edges[0];
        if (q >= s->edges[1]) {
            a = 2;
            q -= s->edges[1];
        }
    }
    uint32_t d[3];
    edge_dims(s, a, d);
    p[0] = (int)(q % d[0]);
    p[1] = (int)((q / d[0]) % d[1]);
    p[2] = (int)(q / (d[0] * d[1]));
    *axis = a;
}
static int boundary(const OEm *s, const int p[3], int axis) {
    int a = (axis + 1) % 3, b = (axis + 2) % 3;
    return p[a] == 0 || (uint32_t)p[a] == s->dims[a] || p[b] == 0 || (uint32_t)p[b] == s->dims[b];
}

/* ---- material coefficients (induction.wgsl:16-31) ---- */
static void cell_properties(OEm *s, const int p[3], float *sigma, float *mu) {
    if (!valid3(p, s->dims) || s->control[2] == 1) {
        *sigma = 0.0f;
        *mu = 1.0f;
        return;
    }
    uint32_t i = (uint32_t)p[0] + s->dims[0] * ((uint32_t)p[1] + s->dims[1] * (uint32_t)p[2]);
    uint32_t id = s->materials[i];
    if (id == 0) {
        *sigma = s->props[0];
        *mu = s->props[1];
        return;
    }
    if (id & 0x80000000u) {
        uint32_t m = id & 255u;
        if (m >= s->n_props) { s->bad_id = 1; *sigma = 0.0f; *mu = 1.0f; return; }
        float alpha = (float)((id >> 8) & 0x7fffffu) / 8388607.0f;
        *sigma = alpha * s->props[2 * m];
        *mu = s->props[1] * (1.0f - alpha) + s->props[2 * m + 1] * alpha;
        return;
    }
    if (id >= s->n_props) { s->bad_id = 1; *sigma = 0.0f; *mu = 1.0f; return; }
    *sigma = s->props[2 * id];
    *mu = s->props[2 * id + 1];
}
static float cell_sigma(OEm *s, const int p[3]) { float a, b; cell_properties(s, p, &a, &b); return a; }
static float cell_mu(OEm *s, const int p[3]) { float a, b; cell_properties(s, p, &a, &b); return b; }

static float nu_face(OEm *s, int axis, const int p[3]) {
    uint32_t d[3];
    face_dims(s, axis, d);
    if (!valid3(p, d)) return 0.0f;
    int q[3] = {p[0], p[1], p[2]};
    q[axis] -= 1;
    return 0.5f / cell_mu(s, p) + 0.5f / cell_mu(s, q);
}

/* kind 0: reaction increment, 1: search direction, 2: applied potential,
   4: accepted reaction, 3: accepted + increment + applied (total). */
static float a_edge(OEm *s, int axis, const int p[3], int kind) {
    uint32_t d[3];
    edge_dims(s, axis, d);
    if (!valid3(p, d)) return 0.0f;
    uint32_t i = edge_index(s, axis, p);
    if (kind == 0) return s->work[i].x;
    if (kind == 1) return s->work[i].z;
    if (kind == 2) return s->source[i].x;
    if (kind == 4) return s->previous[i];
    return s->previous[i] + s->work[i].x + s->source[i].x;
}
static float curl_face(OEm *s, int axis, const int p[3], int kind) {
    uint32_t d[3];
    face_dims(s, axis, d);
    if (!valid3(p, d)) return 0.0f;
    int a = (axis + 1) % 3, b = (axis + 2) % 3;
    int qa[3] = {p[0], p[1], p[2]}, qb[3] = {p[0], p[1], p[2]};
    qa[a] += 1;
    qb[b] += 1;
    return a_edge(s, b, qa, kind) - a_edge(s, b, p, kind) - a_edge(s, a, qb, kind) + a_edge(s, a, p, kind);
}
static float face_term(OEm *s, int axis, const int p[3], int kind, int contrast) {
    uint32_t d[3];
    face_dims(s, axis, d);
    if (!valid3(p, d)) return 0.0f;
    float nu = nu_face(s, axis, p);
    if (contrast) nu = 1.0f - nu;
    return nu * curl_face(s, axis, p, kind);
}
static float adjoint(OEm *s, const int p[3], int w, int kind, int contrast) {
    int a = (w + 1) % 3, b = (w + 2) % 3;
    int qa[3] = {p[0], p[1], p[2]}, qb[3] = {p[0], p[1], p[2]};
    qa[a] -= 1;
    qb[b] -= 1;
    return face_term(s, b, p, kind, contrast) - face_term(s, b, qa, kind, contrast) -
           face_term(s, a, p, kind, contrast) + face_term(s, a, qb, kind, contrast);
}
static int air_node(OEm *s, const int p[3]) {
    for (int k = 0; k < 3; k++)
        if (p[k] <= 0 || p[k] >= (int)s->dims[k]) return 0;
    for (int x = 0; x < 2; x++)
        for (int y = 0; y < 2; y++)
            for (int z = 0; z < 2; z++) {
                int q[3] = {p[0] - x, p[1] - y, p[2] - z};
                if (cell_sigma(s, q) > 0.0f) return 0;
            }
    return 1;
}
static float node_div(OEm *s, const int p[3], int kind) {
    float value = 0.0f;
    for (int a = 0; a < 3; a++) {
        int q[3] = {p[0], p[1], p[2]};
        q[a] -= 1;
        value += a_edge(s, a, p, kind) - a_edge(s, a, q, kind);
    }
    return value;
}
static float gauge(OEm *s, uint32_t i, const int p[3], int w, int kind) {
    f4 flags = s->source[i + s->edges[3]];
    int upper[3] = {p[0], p[1], p[2]};
    upper[w] += 1;
    float value = 0.0f;
    if (flags.y > 0.5f) value += node_div(s, p, kind);
    if (flags.z > 0.5f) value -= node_div(s, upper, kind);
    return value;
}
static float mass(const OEm *s, uint32_t i) {
    if (s->control[1] == 1) return 0.0f;
    return s->physical[1] * s->source[i].z * s->physical[2] * s->physical[2] / s->physical[0];
}
static float diagonal(const OEm *s, uint32_t i) { return maxf(s->source[i].w + mass(s, i), 1e-30f); }
static float residual_scale(const OEm *s) { return s->scalars[6].x > 0.0f ? s->scalars[6].x : 1.0f; }

/* ---- reductions: 256-lane workgroup trees ---- */
enum { RED_SUM = 0, RED_COEF = 1 };
static f4 combine(f4 a, f4 b, int op) {
    if (op == RED_SUM) return add4(a, b);
    return F4(a.x + b.x, minf(a.y, b.y), maxf(a.z, b.z), a.w + b.w);
}
static f4 tree(f4 *lane, int op) {
    for (int st = 128; st > 0; st /= 2)
        for (int l = 0; l < st; l++) lane[l] = combine(lane[l], lane[l + st], op);
    return lane[0];
}
static uint32_t groups_of(uint32_t n) { return (n + 255u) / 256u; }
/* The single-group reduce: lane l accumulates partials l, l+256, ... from
   `init`, then the lanes are combined by the tree. */
static f4 final_reduce(const f4 *partials, uint32_t n, uint32_t stride, f4 init, int op) {
    f4 lane[256];
    for (uint32_t l = 0; l < 256; l++) {
        f4 v = init;
        for (uint32_t i = l; i < n; i += 256) v = combine(v, partials[(size_t)i * stride], op);
        lane[l] = v;
    }
    return tree(lane, op);
}

/* Runs `body` for every edge of each 256-edge group and stores the group's
   tree sum in partials[g]. */
typedef f4 (*edge_fn)(OEm *s, uint32_t i);
static void edge_pass(OEm *s, edge_fn body, f4 init, int op, int store) {
    uint32_t n = s->edges[3], ng = groups_of(n);
#pragma omp parallel for schedule(static)
    for (uint32_t g = 0; g < ng; g++) {
        f4 lane[256];
        for (uint32_t l = 0; l < 256; l++) {
            uint32_t i = g * 256 + l;
            lane[l] = i < n ? body(s, i) : init;
        }
        f4 t = tree(lane, op);
        if (store) s->partials[g] = t;
    }
}

/* ---- passes ---- */
static f4 k_coefficients(OEm *s, uint32_t i) {
    int p[3], w;
    edge_decode(s, i, p, &w);
    int a = (w + 1) % 3, b = (w + 2) % 3;
    f4 v = F4(0.0f, 1e30f, 0.0f, 0.0f);
    float sigma = 0.0f;
    for (int u = 0; u < 2; u++)
        for (int vv = 0; vv < 2; vv++) {
            int q[3] = {p[0], p[1], p[2]};
            q[a] -= u;
            q[b] -= vv;
            sigma += 0.25f * cell_sigma(s, q);
        }
    int qa[3] = {p[0], p[1], p[2]}, qb[3] = {p[0], p[1], p[2]};
    qa[a] -= 1;
    qb[b] -= 1;
    float nb0 = nu_face(s, b, p), nb1 = nu_face(s, b, qa), na0 = nu_face(s, a, p), na1 = nu_face(s, a, qb);
    float diag = nb0 + nb1 + na0 + na1;
    if (boundary(s, p, w)) {
        diag = 1.0f;
        if (sigma > 0.0f) v.x = 1.0f;
    }
    int upper[3] = {p[0], p[1], p[2]};
    upper[w] += 1;
    float lower_air = air_node(s, p) ? 1.0f : 0.0f;
    float upper_air = air_node(s, upper) ? 1.0f : 0.0f;
    int scalar_air = lower_air > 0.5f && upper_air > 0.5f && nb0 == 1.0f && nb1 == 1.0f && na0 == 1.0f && na1 == 1.0f;
    s->source[i + s->edges[3]] = F4(0.0f, lower_air, upper_air, scalar_air ? 1.0f : 0.0f);
    s->source[i].z = sigma;
    s->source[i].w = diag + lower_air + upper_air;
    v.y = sigma > 0.0f ? sigma : 1e30f;
    v.z = sigma;
    v.w = sigma > 0.0f ? 1.0f : 0.0f;
    return v;
}

static f4 k_prepare(OEm *s, uint32_t i) {
    int p[3], w;
    edge_decode(s, i, p, &w);
    uint32_t E = s->edges[3];
    float m = mass(s, i);
    float b = m * s->physical[0] * s->source[i + E].x - m * (s->source[i].x - s->source[i].y) +
              adjoint(s, p, w, 2, 1) - adjoint(s, p, w, 4, 0) - gauge(s, i, p, w, 4);
    float r = b;
    if (s->origin[3] > 0.0f) r -= adjoint(s, p, w, 0, 0) + gauge(s, i, p, w, 0) + m * s->work[i].x;
    if (boundary(s, p, w)) {
        r = 0.0f;
        b = 0.0f;
    }
    float physical_l1 = fabsf(b);
    float scale = residual_scale(s);
    b /= scale;
    r /= scale;
    float z = r / diagonal(s, i);
    s->work[i].y = r;
    s->work[i].z = z;
    s->work[i].w = 0.0f;
    return F4(r * z, r * r, b * b, physical_l1);
}

static void initial_reduce(OEm *s) {
    f4 sum = final_reduce(s->partials, groups_of(s->edges[3]), 1, F4(0, 0, 0, 0), RED_SUM);
    float scale = residual_scale(s), next = scale;
    if (scale == 1.0f && sum.w > 0.0f && (sum.w < 1e-8f || sum.w > 1e8f)) {
        uint32_t bits;
        memcpy(&bits, &sum.w, 4);
        int e = (int)((bits >> 23) & 255u) - 127;
        e = e < -100 ? -100 : e > 100 ? 100 : e;
        uint32_t nb = (uint32_t)(e + 127) << 23;
        memcpy(&next, &nb, 4);
    }
    float absolute_floor = 1e-38f;
    if (scale != 1.0f) {
        float floor_norm = 1e-19f / scale;
        absolute_floor = floor_norm * floor_norm;
    }
    float threshold = sum.z * s->physical[3] + absolute_floor;
    s->scalars[6].x = next;
    s->scalars[0] = F4(sum.x, sum.y, sum.z, threshold);
    s->scalars[1] = F4(next != scale ? next : 0.0f, 0.0f, 0.0f, sum.y <= threshold ? 1.0f : 0.0f);
}

static float air_laplacian(const OEm *s, uint32_t i) {
    int axis = 0;
    if (i >= s->edges[0]) {
        axis = 1;
        if (i >= s->edges[0] + s->edges[1]) axis = 2;
    }
    uint32_t d[3];
    edge_dims(s, axis, d);
    uint32_t zs = d[0] * d[1];
    const f4 *wk = s->work;
    float c = wk[i].z, result = 0.0f;
    result += (c - wk[i - 1].z) + (c - wk[i + 1].z);
    result += (c - wk[i - d[0]].z) + (c - wk[i + d[0]].z);
    result += (c - wk[i - zs].z) + (c - wk[i + zs].z);
    return result;
}

static int g_use_air = 1; /* cleared only by oem_apply_operator's comparison mode */
static f4 k_apply(OEm *s, uint32_t i) {
    float dot = 0.0f;
    if (s->scalars[1].w == 0.0f) {
        float q;
        if (g_use_air && s->source[i + s->edges[3]].w > 0.5f) {
            q = air_laplacian(s, i);
        } else {
            int p[3], w;
            edge_decode(s, i, p, &w);
            q = adjoint(s, p, w, 1, 0) + gauge(s, i, p, w, 1) + mass(s, i) * s->work[i].z;
            if (boundary(s, p, w)) q = s->work[i].z;
        }
        s->work[i].w = q;
        dot = s->work[i].z * q;
    }
    return F4(dot, 0.0f, 0.0f, 0.0f);
}

static void alpha_reduce(OEm *s) {
    f4 sum = final_reduce(s->partials, groups_of(s->edges[3]), 1, F4(0, 0, 0, 0), RED_SUM);
    if (s->scalars[1].w == 0.0f) {
        if (sum.x <= 0.0f || fabsf(sum.x) > 3e38f) s->scalars[1].w = 2.0f;
        else s->scalars[1].x = s->scalars[0].x / sum.x;
    }
}

static f4 k_update_residual(OEm *s, uint32_t i) {
    f4 v = F4(0, 0, 0, 0);
    if (s->scalars[1].w == 0.0f) {
        f4 old = s->work[i];
        float alpha = s->scalars[1].x;
        float r = old.y - alpha * old.w;
        float d = diagonal(s, i);
        s->work[i] = F4(old.x + residual_scale(s) * (alpha * old.z), r, old.z, d);
        v = F4(r * r / d, r * r, 0.0f, 0.0f);
    }
    return v;
}

static void beta_reduce(OEm *s) {
    f4 sum = final_reduce(s->partials, groups_of(s->edges[3]), 1, F4(0, 0, 0, 0), RED_SUM);
    if (s->scalars[1].w == 0.0f) {
        s->scalars[1].y = sum.x / s->scalars[0].x;
        s->scalars[0].x = sum.x;
        s->scalars[0].y = sum.y;
        s->scalars[1].z += 1.0f;
        if (sum.y <= s->scalars[0].w) s->scalars[1].w = 1.0f;
        if (fabsf(sum.x) > 3e38f || fabsf(sum.y) > 3e38f) s->scalars[1].w = 2.0f;
    }
}

static void update_search(OEm *s) {
    if (s->scalars[1].w != 0.0f) return;
    float beta = s->scalars[1].y;
#pragma omp parallel for schedule(static)
    for (uint32_t i = 0; i < s->edges[3]; i++) {
        f4 v = s->work[i];
        float z = v.w;
        if (s->control[3] != 1) z = v.y / v.w;
        s->work[i].z = z + beta * v.z;
    }
}

static f4 k_true_residual(OEm *s, uint32_t i) {
    int p[3], w;
    edge_decode(s, i, p, &w);
    uint32_t E = s->edges[3];
    float m = mass(s, i);
    float r = m * s->physical[0] * s->source[i + E].x - m * (s->work[i].x + (s->source[i].x - s->source[i].y)) +
              adjoint(s, p, w, 2, 1) - adjoint(s, p, w, 4, 0) - gauge(s, i, p, w, 4) - adjoint(s, p, w, 0, 0) -
              gauge(s, i, p, w, 0);
    if (boundary(s, p, w)) r = 0.0f;
    r /= residual_scale(s);
    float d = diagonal(s, i);
    s->work[i].y = r;
    s->work[i].z = r / d;
    return F4(r * r / d, r * r, 0.0f, 0.0f);
}

static void restart_reduce(OEm *s) {
    f4 sum = final_reduce(s->partials, groups_of(s->edges[3]), 1, F4(0, 0, 0, 0), RED_SUM);
    s->scalars[0].x = sum.x;
    s->scalars[0].y = sum.y;
    s->scalars[1].w = sum.y <= s->scalars[0].w ? 1.0f : 0.0f;
}

/* ---- nodal gradient-space correction (src/em/nodal.wgsl) ---- */
static uint32_t nodal_count(const OEm *s) { return (s->dims[0] + 1) * (s->dims[1] + 1) * (s->dims[2] + 1); }
static float cached_air_node(const OEm *s, const int p[3]) {
    for (int k = 0; k < 3; k++)
        if (p[k] <= 0 || p[k] >= (int)s->dims[k]) return 0.0f;
    return s->source[edge_index(s, 0, p) + s->edges[3]].y;
}
static float nodal_value(const OEm *s, uint32_t i) {
    uint32_t d0 = s->dims[0] + 1, d1 = s->dims[1] + 1;
    int p[3] = {(int)(i % d0), (int)((i / d0) % d1), (int)(i / (d0 * d1))};
    for (int k = 0; k < 3; k++)
        if (p[k] <= 0 || p[k] >= (int)s->dims[k]) return 0.0f;
    float rhs = 0.0f, diag = 36.0f * cached_air_node(s, p);
    for (int a = 0; a < 3; a++) {
        int lower[3] = {p[0], p[1], p[2]}, upper[3] = {p[0], p[1], p[2]};
        lower[a] -= 1;
        upper[a] += 1;
        uint32_t out = edge_index(s, a, p), inc = edge_index(s, a, lower);
        rhs += s->work[out].y - s->work[inc].y;
        diag += mass(s, out) + mass(s, inc) + cached_air_node(s, lower) + cached_air_node(s, upper);
    }
    return rhs / maxf(diag, 1e-30f);
}
static void nodal_build(OEm *s, int initial) {
    if (!initial && s->scalars[1].w != 0.0f) return;
    uint32_t n = nodal_count(s);
#pragma omp parallel for schedule(static)
    for (uint32_t i = 0; i < n; i++) s->nodal[i] = nodal_value(s, i);
}
static float nodal_z(const OEm *s, uint32_t i) {
    int p[3], w;
    edge_decode(s, i, p, &w);
    uint32_t d0 = s->dims[0] + 1, d1 = s->dims[1] + 1;
    uint32_t lo = (uint32_t)p[0] + d0 * ((uint32_t)p[1] + d1 * (uint32_t)p[2]);
    p[w] += 1;
    uint32_t up = (uint32_t)p[0] + d0 * ((uint32_t)p[1] + d1 * (uint32_t)p[2]);
    return s->work[i].y / diagonal(s, i) + s->nodal[lo] - s->nodal[up];
}
static int g_nodal_initial = 0;
static f4 k_nodal(OEm *s, uint32_t i) {
    f4 v = F4(0, 0, 0, 0);
    if (g_nodal_initial) {
        float r = s->work[i].y, z = nodal_z(s, i);
        s->work[i].z = z;
        s->work[i].w = z;
        v = F4(r * z, r * r, 0.0f, 0.0f);
    } else if (s->scalars[1].w == 0.0f) {
        float r = s->work[i].y, z = nodal_z(s, i);
        s->work[i].w = z;
        v = F4(r * z, r * r, 0.0f, 0.0f);
    }
    return v;
}
/* nodal_initial / nodal_update: only the x and y lanes of the partials are
   written (the update only while the solve is active). */
static void nodal_pass(OEm *s, int initial) {
    uint32_t n = s->edges[3], ng = groups_of(n);
    int write = initial || s->scalars[1].w == 0.0f;
    g_nodal_initial = initial;
#pragma omp parallel for schedule(static)
    for (uint32_t g = 0; g < ng; g++) {
        f4 lane[256];
        for (uint32_t l = 0; l < 256; l++) {
            uint32_t i = g * 256 + l;
            lane[l] = i < n ? k_nodal(s, i) : F4(0, 0, 0, 0);
        }
        f4 t = tree(lane, RED_SUM);
        if (write) {
            s->partials[g].x = t.x;
            s->partials[g].y = t.y;
        }
    }
}
/* append_nodal (src/em/mod.rs:639-659) */
static void append_nodal(OEm *s, int initial) {
    if (s->control[3] != 1) return;
    nodal_build(s, initial);
    nodal_pass(s, initial);
}

static void begin_step(OEm *s) {
    s->scalars[6].x = 1.0f;
#pragma omp parallel for schedule(static)
    for (uint32_t i = 0; i < s->edges[3]; i++) {
        float accepted = s->work[i].x, guess = 0.0f;
        int p[3], w;
        edge_decode(s, i, p, &w);
        if (s->origin[3] > 0.0f && !boundary(s, p, w)) guess = s->origin[3] * (accepted - s->previous[i]);
        s->previous[i] = accepted;
        s->work[i].x = guess;
    }
}
static void zero_guess(OEm *s) {
    for (uint32_t i = 0; i < s->edges[3]; i++) s->work[i].x = 0.0f;
}
static void commit_step(OEm *s) {
    for (uint32_t i = 0; i < s->edges[3]; i++) s->work[i].x += s->previous[i];
}
static void rollback(OEm *s) {
    for (uint32_t i = 0; i < s->edges[3]; i++) {
        s->work[i].x = s->previous[i];
        s->source[i].x = s->source[i].y;
    }
}

/* fields (induction.wgsl:188-216) */
static float electric_edge(OEm *s, int axis, const int p[3]) {
    uint32_t d[3];
    edge_dims(s, axis, d);
    if (s->control[1] == 1 || !valid3(p, d)) return 0.0f;
    uint32_t i = edge_index(s, axis, p);
    return -(s->work[i].x + (s->source[i].x - s->source[i].y)) / s->physical[0] + s->source[i + s->edges[3]].x;
}
static float current_edge(OEm *s, int axis, const int p[3]) {
    uint32_t d[3];
    edge_dims(s, axis, d);
    if (!valid3(p, d)) return 0.0f;
    return s->source[edge_index(s, axis, p)].z * electric_edge(s, axis, p);
}
static float len3(float x, float y, float z) { return sqrtf(x * x + y * y + z * z); }

static void fields_cell(OEm *s, uint32_t i, f4 out[4]) {
    uint32_t nx = s->dims[0], ny = s->dims[1];
    int p[3] = {(int)(i % nx), (int)((i / nx) % ny), (int)(i / (nx * ny))};
    float sig, mu;
    cell_properties(s, p, &sig, &mu);
    float h = s->physical[2];
    float mag[3] = {0, 0, 0}, app[3] = {0, 0, 0}, j[3] = {0, 0, 0};
    float heat = 0.0f, div_b = 0.0f, div_j = 0.0f, max_edge = 0.0f, msq = 0.0f;
    for (int axis = 0; axis < 3; axis++) {
        int upper[3] = {p[0], p[1], p[2]};
        upper[axis] += 1;
        float b0 = curl_face(s, axis, p, 3) / h, b1 = curl_face(s, axis, upper, 3) / h;
        msq += 0.5f * (b0 * b0 + b1 * b1);
        mag[axis] = 0.5f * (b0 + b1);
        app[axis] = 0.5f * (curl_face(s, axis, p, 2) + curl_face(s, axis, upper, 2)) / h;
        div_b += b1 - b0;
        int aa = (axis + 1) % 3, bb = (axis + 2) % 3;
        float es = 0.0f;
        for (int u = 0; u < 2; u++)
            for (int v = 0; v < 2; v++) {
                int q[3] = {p[0], p[1], p[2]};
                q[aa] += u;
                q[bb] += v;
                float ee = electric_edge(s, axis, q);
                es += 0.25f * ee;
                heat += sig * 0.25f * ee * ee;
            }
        j[axis] = sig * es;
        int prev[3] = {p[0], p[1], p[2]};
        prev[axis] -= 1;
        float jp = current_edge(s, axis, p), jm = current_edge(s, axis, prev);
        div_j += jp - jm;
        max_edge = maxf(max_edge, maxf(fabsf(jp), fabsf(jm)));
    }
    float f[3] = {j[1] * mag[2] - j[2] * mag[1], j[2] * mag[0] - j[0] * mag[2], j[0] * mag[1] - j[1] * mag[0]};
    float bn = len3(mag[0], mag[1], mag[2]), jn = len3(j[0], j[1], j[2]), fn = len3(f[0], f[1], f[2]);
    float vol = h * h * h;
    float an = len3(app[0], app[1], app[2]);
    s->results[4 * (size_t)i + 0] = F4(mag[0], mag[1], mag[2], bn);
    s->results[4 * (size_t)i + 1] = F4(j[0], j[1], j[2], jn);
    s->results[4 * (size_t)i + 2] = F4(f[0], f[1], f[2], heat);
    s->results[4 * (size_t)i + 3] = F4(app[0], app[1], app[2], an);
    out[0] = F4(bn, jn, fn, heat);
    out[1] = F4(f[0] * vol, f[1] * vol, f[2] * vol, heat * vol);
    out[2] = F4(fabsf(div_j), max_edge, fabsf(div_b), msq * vol / (2.0f * s->physical[1] * mu));
    out[3] = F4(an, len3(mag[0] - app[0], mag[1] - app[1], mag[2] - app[2]), 0.0f, 0.0f);
}
static f4 max4(f4 a, f4 b) { return F4(maxf(a.x, b.x), maxf(a.y, b.y), maxf(a.z, b.z), maxf(a.w, b.w)); }
static f4 cmix(f4 a, f4 b) { return F4(maxf(a.x, b.x), maxf(a.y, b.y), maxf(a.z, b.z), a.w + b.w); }
static void fields_tree(f4 la[256], f4 lb[256], f4 lc[256], f4 ld[256], f4 out[4]) {
    for (int st = 128; st > 0; st /= 2)
        for (int l = 0; l < st; l++) {
            la[l] = max4(la[l], la[l + st]);
            lb[l] = add4(lb[l], lb[l + st]);
            lc[l] = cmix(lc[l], lc[l + st]);
            ld[l] = max4(ld[l], ld[l + st]);
        }
    out[0] = la[0];
    out[1] = lb[0];
    out[2] = lc[0];
    out[3] = ld[0];
}
static void fields(OEm *s) {
    uint32_t n = s->dims[3], ng = groups_of(n);
#pragma omp parallel for schedule(static)
    for (uint32_t g = 0; g < ng; g++) {
        f4 la[256], lb[256], lc[256], ld[256], o[4];
        for (uint32_t l = 0; l < 256; l++) {
            uint32_t i = g * 256 + l;
            if (i < n) {
                fields_cell(s, i, o);
                la[l] = o[0]; lb[l] = o[1]; lc[l] = o[2]; ld[l] = o[3];
            } else {
                la[l] = lb[l] = lc[l] = ld[l] = F4(0, 0, 0, 0);
            }
        }
        fields_tree(la, lb, lc, ld, o);
        for (int k = 0; k < 4; k++) s->partials[4 * (size_t)g + k] = o[k];
    }
}
static void field_reduce(OEm *s) {
    uint32_t n = groups_of(s->dims[3]);
    f4 la[256], lb[256], lc[256], ld[256], o[4];
    for (uint32_t l = 0; l < 256; l++) {
        f4 a = F4(0, 0, 0, 0), b = a, c = a, d = a;
        for (uint32_t i = l; i < n; i += 256) {
            f4 v = s->partials[4 * (size_t)i + 2];
            a = max4(a, s->partials[4 * (size_t)i]);
            b = add4(b, s->partials[4 * (size_t)i + 1]);
            c = F4(maxf(c.x, v.x), maxf(c.y, v.y), maxf(c.z, v.z), c.w + v.w);
            d = max4(d, s->partials[4 * (size_t)i + 3]);
        }
        la[l] = a; lb[l] = b; lc[l] = c; ld[l] = d;
    }
    fields_tree(la, lb, lc, ld, o);
    for (int k = 0; k < 4; k++) s->scalars[2 + k] = o[k];
}

/* ---- public entry points (mhd_oracle.h) ---- */
OEm *oem_new(const uint32_t dims[3], float h, const float origin[3], double dt_s, float rel_tol, uint32_t max_it,
             int vacuum) {
    OEm *s = (OEm *)calloc(1, sizeof(OEm));
    if (!s) return NULL;
    uint64_t x = dims[0], y = dims[1], z = dims[2];
    s->dims[0] = dims[0]; s->dims[1] = dims[1]; s->dims[2] = dims[2];
    s->dims[3] = (uint32_t)(x * y * z);
    s->edges[0] = (uint32_t)(x * (y + 1) * (z + 1));
    s->edges[1] = (uint32_t)((x + 1) * y * (z + 1));
    s->edges[2] = (uint32_t)((x + 1) * (y + 1) * z);
    s->edges[3] = s->edges[0] + s->edges[1] + s->edges[2];
    s->control[2] = vacuum ? 1u : 0u;
    s->control[1] = 1u;
    for (int k = 0; k < 3; k++) s->origin[k] = origin[k];
    s->physical[0] = 1e-5f;
    s->physical[1] = 4e-7f * 3.14159265358979323846f;
    s->physical[2] = h;
    s->physical[3] = 1e-10f;
    s->dt_s = dt_s;
    s->rel_tol = rel_tol;
    s->max_it = max_it;
    size_t E = s->edges[3], C = s->dims[3];
    size_t ng = groups_of((uint32_t)(E > C ? E : C));
    s->materials = (uint32_t *)calloc(C ? C : 1, 4);
    s->source = (f4 *)calloc(2 * E, sizeof(f4));
    s->work = (f4 *)calloc(E, sizeof(f4));
    s->previous = (float *)calloc(E, 4);
    s->partials = (f4 *)calloc(4 * ng + 4, sizeof(f4));
    s->results = (f4 *)calloc(4 * C + 4, sizeof(f4));
    s->checkpoint = (f4 *)calloc(4 * C + 4, sizeof(f4));
    s->nodal = (float *)calloc((size_t)(x + 1) * (y + 1) * (z + 1), 4);
    s->nodal_after = 1024;
    if (!s->materials || !s->source || !s->work || !s->previous || !s->partials || !s->results || !s->checkpoint ||
        !s->nodal) {
        oem_free(s);
        return NULL;
    }
    return s;
}

void oem_free(OEm *s) {
    if (!s) return;
    free(s->materials); free(s->props); free(s->source); free(s->work); free(s->previous);
    free(s->partials); free(s->results); free(s->checkpoint); free(s->nodal);
    free(s);
}

void oem_sizes(const OEm *s, uint32_t out[8]) {
    for (int k = 0; k < 4; k++) { out[k] = s->dims[k]; out[4 + k] = s->edges[k]; }
}

/* coefficients + coefficient_check (induction.wgsl:105-130).  Returns 0, or
   -1 when a material id has no property row. */
int oem_set_materials(OEm *s, const uint32_t *materials, const float *props, uint32_t n_props, float check[4]) {
    memcpy(s->materials, materials, (size_t)s->dims[3] * 4);
    free(s->props);
    s->props = (float *)malloc((size_t)(n_props ? n_props : 1) * 2 * 4);
    memcpy(s->props, props, (size_t)n_props * 2 * 4);
    s->n_props = n_props;
    s->bad_id = 0;
    edge_pass(s, k_coefficients, F4(0.0f, 1e30f, 0.0f, 0.0f), RED_COEF, 1);
    f4 c = final_reduce(s->partials, groups_of(s->edges[3]), 1, F4(0.0f, 1e30f, 0.0f, 0.0f), RED_COEF);
    s->scalars[0] = c;
    check[0] = c.x; check[1] = c.y; check[2] = c.z; check[3] = c.w;
    return s->bad_id ? -1 : 0;
}

void oem_set_motional(OEm *s, const float *emf) {
    for (uint32_t i = 0; i < s->edges[3]; i++) s->source[i + s->edges[3]].x = emf ? emf[i] : 0.0f;
}
/* energy ledger (src/em/energy.wgsl, EmState::energy_step mod.rs:1106-1133),
   after a step is committed.  kind 0: new total potential (reaction +
   applied), 1: previous total, 3: its increment, 2: applied potential. */
static float en_a(const OEm *s, int axis, const int p[3], int kind) {
    uint32_t d[3];
    edge_dims(s, axis, d);
    if (!valid3(p, d)) return 0.0f;
    uint32_t i = edge_index(s, axis, p);
    if (kind == 0) return s->work[i].x + s->source[i].x;
    if (kind == 1) return s->previous[i] + s->source[i].y;
    if (kind == 3) return (s->work[i].x - s->previous[i]) + (s->source[i].x - s->source[i].y);
    return s->source[i].x;
}
static float en_curl(const OEm *s, int axis, const int p[3], int kind) {
    uint32_t d[3];
    face_dims(s, axis, d);
    if (!valid3(p, d)) return 0.0f;
    int a = (axis + 1) % 3, b = (axis + 2) % 3;
    int qa[3] = {p[0], p[1], p[2]}, qb[3] = {p[0], p[1], p[2]};
    qa[a] += 1;
    qb[b] += 1;
    return en_a(s, b, qa, kind) - en_a(s, b, p, kind) - en_a(s, a, qb, kind) + en_a(s, a, p, kind);
}
static float en_face(OEm *s, int axis, const int p[3], int kind, int weighted) {
    uint32_t d[3];
    face_dims(s, axis, d);
    if (!valid3(p, d)) return 0.0f;
    return en_curl(s, axis, p, kind) * (weighted ? nu_face(s, axis, p) : 1.0f);
}
static float en_adjoint(OEm *s, const int p[3], int w, int kind, int weighted) {
    int a = (w + 1) % 3, b = (w + 2) % 3;
    int qa[3] = {p[0], p[1], p[2]}, qb[3] = {p[0], p[1], p[2]};
    qa[a] -= 1;
    qb[b] -= 1;
    return en_face(s, b, p, kind, weighted) - en_face(s, b, qa, kind, weighted) - en_face(s, a, p, kind, weighted) +
           en_face(s, a, qb, kind, weighted);
}
static void energy_item(OEm *s, uint32_t i, f4 *A, f4 *B) {
    float h = s->physical[2], dt = s->physical[0], mu0 = s->physical[1], volume = h * h * h;
    uint32_t E = s->edges[3];
    f4 a = F4(0, 0, 0, 0), b = F4(0, 0, 0, 0);
    if (i < E) {
        int p[3], w;
        edge_decode(s, i, p, &w);
        float delta = (s->work[i].x - s->previous[i]) + (s->source[i].x - s->source[i].y);
        float motion = s->source[i + E].x;
        float ee = -delta / dt + motion;
        float j = s->source[i].z * ee;
        a.w = dt * volume * j * ee;
        b.x = -dt * volume * j * motion;
        float drive = en_adjoint(s, p, w, 2, 0);
        if (boundary(s, p, w)) drive = en_adjoint(s, p, w, 0, 1);
        b.y = h / mu0 * delta * drive;
    }
    uint32_t nx = s->dims[0], ny = s->dims[1], nz = s->dims[2];
    uint32_t fx = (nx + 1) * ny * nz, fy = nx * (ny + 1) * nz, fz = nx * ny * (nz + 1);
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
        uint32_t d[3];
        face_dims(s, axis, d);
        int p[3] = {(int)(q % d[0]), (int)((q / d[0]) % d[1]), (int)(q / (d[0] * d[1]))};
        float now = en_curl(s, axis, p, 0), old = en_curl(s, axis, p, 1), dl = en_curl(s, axis, p, 3);
        float scale = h / (2.0f * mu0) * nu_face(s, axis, p);
        a.x = scale * now * now;
        a.y = scale * dl * (now + old);
        a.z = scale * dl * dl;
    }
    *A = a;
    *B = b;
}
/* out: magnetic, delta magnetic, backward-Euler loss, Joule, mechanical,
   external work, balance error (J); returns -1 for a non-finite integral. */
int oem_energy(OEm *s, double out[7]) {
    uint32_t n = s->edges[3], ng = groups_of(n);
    f4 *pa = (f4 *)calloc(2 * (size_t)ng + 2, sizeof(f4));
#pragma omp parallel for schedule(static)
    for (uint32_t g = 0; g < ng; g++) {
        f4 la[256], lb[256];
        for (uint32_t l = 0; l < 256; l++) energy_item(s, g * 256 + l, &la[l], &lb[l]);
        for (int st = 128; st > 0; st /= 2)
            for (int l = 0; l < st; l++) {
                la[l] = add4(la[l], la[l + st]);
                lb[l] = add4(lb[l], lb[l + st]);
            }
        pa[g] = la[0];
        pa[ng + g] = lb[0];
    }
    f4 A = final_reduce(pa, ng, 1, F4(0, 0, 0, 0), RED_SUM);
    f4 B = final_reduce(pa + ng, ng, 1, F4(0, 0, 0, 0), RED_SUM);
    free(pa);
    float v[8] = {A.x, A.y, A.z, A.w, B.x, B.y, B.z, B.w};
    for (int k = 0; k < 8; k++)
        if (!isfinite(v[k])) return -1;
    for (int k = 0; k < 6; k++) out[k] = v[k];
    out[6] = 0.0;
    if (s->time_s == 0.0) {
        for (int k = 1; k < 7; k++) out[k] = 0.0;
        return 0;
    }
    out[6] = out[5] - out[1] - out[2] - out[3] - out[4];
    return 0;
}

/* body integrals (src/em/body-stats.wgsl): for each body z (< 32) the force
   and Joule power, sum over the cells with bit z of masks[i] of
   ((fq * h) * h) * h, as 256-cell group trees and a 256-stride final pass. */
void oem_body_forces(const OEm *s, const uint32_t *masks, uint32_t bodies, float *totals) {
    uint32_t n = s->dims[3], ng = groups_of(n);
    float h = s->physical[2];
    f4 *part = (f4 *)calloc((size_t)ng + 1, sizeof(f4));
    for (uint32_t z = 0; z < bodies; z++) {
        for (uint32_t g = 0; g < ng; g++) {
            f4 lane[256];
            for (uint32_t l = 0; l < 256; l++) {
                uint32_t i = g * 256 + l;
                f4 v = F4(0, 0, 0, 0);
                if (i < n && (masks[i] & (1u << z))) {
                    f4 q = s->results[4 * (size_t)i + 2];
                    v = F4(q.x * h * h * h, q.y * h * h * h, q.z * h * h * h, q.w * h * h * h);
                }
                lane[l] = v;
            }
            part[g] = tree(lane, RED_SUM);
        }
        f4 t = final_reduce(part, ng, 1, F4(0, 0, 0, 0), RED_SUM);
        totals[4 * z + 0] = t.x;
        totals[4 * z + 1] = t.y;
        totals[4 * z + 2] = t.z;
        totals[4 * z + 3] = t.w;
    }
    free(part);
}

/* source pass (src/em/source.wgsl:5-17): the applied potential of the
   source elements at every edge midpoint, summed in batches of 32 elements
   (one pass each in the reference) whose per-batch vector is added to the
   running value.  Element = 12 floats (a, b, c as vec4): c.y < 0.5 a wire
   segment a->b with core radius c.x and current c.z; c.y < 1.5 a surface
   current element at a with moment b scaled by c.z and softening c.x;
   otherwise a uniform field b scaled by c.z.  ash(x) = sign(x) log(|x| +
   sqrt(x^2 + 1)); inverseSqrt(x) = 1/sqrtf(x). */
static float ash(float x) {
    float sg = x > 0.0f ? 1.0f : x < 0.0f ? -1.0f : 0.0f;
    return sg * logf(fabsf(x) + sqrtf(x * x + 1.0f));
}
void oem_evaluate_sources(const OEm *s, const float *el, uint32_t count, float *out) {
    uint32_t E = s->edges[3];
#pragma omp parallel for schedule(static)
    for (uint32_t i = 0; i < E; i++) {
        int e[3], w;
        edge_decode(s, i, e, &w);
        float pe[3] = {(float)e[0], (float)e[1], (float)e[2]};
        pe[w] += 0.5f;
        float p[3];
        for (int k = 0; k < 3; k++) p[k] = s->origin[k] + pe[k] * s->physical[2];
        float acc = 0.0f;
        uint32_t nb = count == 0 ? 1 : (count + 31) / 32;
        for (uint32_t bi = 0; bi < nb; bi++) {
            uint32_t begin = bi * 32, end = begin + 32 < count ? begin + 32 : count;
            float a = 0.0f;
            for (uint32_t j = begin; j < end; j++) {
                const float *q = el + 12 * (size_t)j;
                const float *A = q, *B = q + 4, *Cc = q + 8;
                if (Cc[2] == 0.0f) continue;
                float r[3] = {p[0] - A[0], p[1] - A[1], p[2] - A[2]};
                if (Cc[1] < 0.5f) {
                    float d[3] = {B[0] - A[0], B[1] - A[1], B[2] - A[2]};
                    float len = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                    float u[3] = {d[0] / len, d[1] / len, d[2] / len};
                    float t = r[0] * u[0] + r[1] * u[1] + r[2] * u[2];
                    float pp[3] = {r[0] - u[0] * t, r[1] - u[1] * t, r[2] - u[2] * t};
                    float radius = sqrtf(pp[0] * pp[0] + pp[1] * pp[1] + pp[2] * pp[2] + Cc[0] * Cc[0]);
                    a += u[w] * (1e-7f * Cc[2] * (ash(t / radius) - ash((t - len) / radius)));
                } else if (Cc[1] < 1.5f) {
                    a += B[w] * (1e-7f * Cc[2] * (1.0f / sqrtf(r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + Cc[0] * Cc[0])));
                } else {
                    float cr[3] = {B[1] * p[2] - B[2] * p[1], B[2] * p[0] - B[0] * p[2], B[0] * p[1] - B[1] * p[0]};
                    a += 0.5f * Cc[2] * cr[w];
                }
            }
            acc = bi == 0 ? a : acc + a;
        }
        out[i] = acc;
    }
}

/* motion (src/em/motion.wgsl:8-26): fluid cell records (16 floats: velocity
   0-2, mobile where float 12 > 0.5) and this state's last B. */
void oem_set_motion(OEm *s, const float *fluid) {
    uint32_t E = s->edges[3];
    for (uint32_t i = 0; i < E; i++) {
        int p[3], w;
        edge_decode(s, i, p, &w);
        int a = (w + 1) % 3, b = (w + 2) % 3;
        float weighted = 0.0f, sigma = 0.0f;
        for (int u = 0; u < 2; u++)
            for (int v = 0; v < 2; v++) {
                int q[3] = {p[0], p[1], p[2]};
                q[a] -= u;
                q[b] -= v;
                if (!valid3(q, s->dims)) continue;
                uint32_t c = (uint32_t)q[0] + s->dims[0] * ((uint32_t)q[1] + s->dims[1] * (uint32_t)q[2]);
                float sc = cell_sigma(s, q);
                sigma += sc;
                const float *f = fluid + (size_t)c * 16;
                if (f[12] > 0.5f) {
                    f4 B = s->results[4 * (size_t)c];
                    float cr[3] = {f[1] * B.z - f[2] * B.y, f[2] * B.x - f[0] * B.z, f[0] * B.y - f[1] * B.x};
                    weighted += sc * cr[w];
                }
            }
        s->source[i + E].x = weighted / maxf(sigma, 1e-30f);
    }
}

void oem_set_reaction(OEm *s, const float *a) {
    for (uint32_t i = 0; i < s->edges[3]; i++) s->work[i].x = a[i];
}
/* which: 0 work (E x 4), 1 previous (E), 2 source (2E x 4), 3 results
   (cells x 16), 4 scalars (32). */
void oem_get(const OEm *s, int which, float *out) {
    size_t E = s->edges[3], C = s->dims[3];
    if (which == 0) memcpy(out, s->work, E * 16);
    else if (which == 1) memcpy(out, s->previous, E * 4);
    else if (which == 2) memcpy(out, s->source, 2 * E * 16);
    else if (which == 3) memcpy(out, s->results, C * 64);
    else memcpy(out, s->scalars, 8 * 16);
}

/* apply_operator on a caller-supplied search direction (the check of
   tests.rs:666-738): q = A p, with or without the air stencil. */
void oem_apply_operator(OEm *s, const float *p, float *q, int use_air) {
    for (uint32_t i = 0; i < s->edges[3]; i++) s->work[i].z = p[i];
    memset(s->scalars, 0, sizeof(s->scalars));
    g_use_air = use_air;
    edge_pass(s, k_apply, F4(0, 0, 0, 0), RED_SUM, 1);
    g_use_air = 1;
    for (uint32_t i = 0; i < s->edges[3]; i++) q[i] = s->work[i].w;
}

static int status_finite(const f4 *sc) {
    const float *v = &sc[0].x;
    for (int k = 0; k < 8; k++)
        if (!isfinite(v[k])) return 0;
    return 1;
}
static void solve_prepare(OEm *s) {
    edge_pass(s, k_prepare, F4(0, 0, 0, 0), RED_SUM, 1);
    append_nodal(s, 1);
    initial_reduce(s);
}
static void restart(OEm *s) {
    edge_pass(s, k_true_residual, F4(0, 0, 0, 0), RED_SUM, 1);
    append_nodal(s, 1);
    restart_reduce(s);
}

void oem_set_nodal_switch(OEm *s, uint32_t after) { s->nodal_after = after; }
void oem_update_config(OEm *s, double dt_s, float rel_tol, uint32_t max_it) {
    s->dt_s = dt_s;
    s->rel_tol = rel_tol;
    s->max_it = max_it;
}
void oem_set_predict(OEm *s, int on) { s->no_predict = !on; }
/* B r with the nodal correction (append_nodal's initial passes on a
   residual r in work.y): out = the preconditioned residual it leaves in
   work.w.  Uses the mass terms of the last step. */
void oem_apply_nodal(OEm *s, const float *r, float *out) {
    uint32_t E = s->edges[3];
    for (uint32_t i = 0; i < E; i++) s->work[i] = F4(0.0f, r[i], 0.0f, 0.0f);
    uint32_t saved = s->control[3];
    s->control[3] = 1;
    append_nodal(s, 1);
    s->control[3] = saved;
    for (uint32_t i = 0; i < E; i++) out[i] = s->work[i].w;
}
void oem_set_previous(OEm *s, const float *a) { memcpy(s->previous, a, (size_t)s->edges[3] * 4); }
void oem_prediction(const OEm *s, float out[3]) { memcpy(out, s->prediction, sizeof s->prediction); }
void oem_time(const OEm *s, double out[2]) {
    out[0] = s->time_s;
    out[1] = s->last_dt;
}

/* EmState::advance_to (src/em/mod.rs:863-1090) for one step to `time_s`.
   `applied` (E floats) is the applied potential at that time, or NULL when it
   is unchanged (hold_source).  status_out: scalars[0..1]; stats_out:
   scalars[2..5].  Returns an OEM_* code. */
int oem_advance(OEm *s, double time_s, int initial, const float *applied, float status_out[8], float stats_out[16]) {
    uint32_t E = s->edges[3];
    s->control[1] = initial ? 1u : 0u;
    float pf = 0.0f;
    if (!s->no_predict && !initial && s->can_predict && s->last_dt > 0.0) {
        float ratio = (float)((time_s - s->time_s) / s->last_dt);
        pf = (isfinite(ratio) && ratio > 0.0f) ? ratio : 0.0f;
    }
    s->origin[3] = pf;
    s->physical[0] = (float)s->dt_s;
    s->physical[3] = s->rel_tol * s->rel_tol;
    int allow_nodal = !initial && s->control[2] == 0 && s->max_it > s->nodal_after;
    /* update_sources leaves control.w = 0; a zero switch point starts in
       nodal mode (src/em/mod.rs:897-903) */
    s->control[3] = (allow_nodal && s->nodal_after == 0) ? 1u : 0u;
    /* update_sources: the source pass shifts the history (source.wgsl:16-17);
       an unchanged field keeps a zero history delta (hold_source). */
    for (uint32_t i = 0; i < E; i++) {
        if (applied) {
            s->source[i].y = s->source[i].x;
            s->source[i].x = applied[i];
            if (initial) s->source[i].y = s->source[i].x;
        } else {
            s->source[i].y = s->source[i].x;
        }
    }
    begin_step(s);
    solve_prepare(s);
    if (s->scalars[1].x != 0.0f) solve_prepare(s);
    s->prediction[0] = pf;
    s->prediction[1] = sqrtf(s->scalars[0].y / maxf(s->scalars[0].z, 1e-38f));
    s->prediction[2] = 0.0f;
    if (pf > 0.0f && (!status_finite(s->scalars) || s->scalars[0].y > s->scalars[0].z)) {
        s->prediction[2] = 1.0f;
        s->origin[3] = 0.0f;
        zero_guess(s);
        solve_prepare(s);
    }
    for (;;) {
        while (s->scalars[1].w == 0.0f && status_finite(s->scalars) && (uint32_t)s->scalars[1].z < s->max_it) {
            uint32_t batch = s->max_it - (uint32_t)s->scalars[1].z;
            if (batch > 32) batch = 32;
            for (uint32_t k = 0; k < batch; k++) {
                edge_pass(s, k_apply, F4(0, 0, 0, 0), RED_SUM, 1);
                alpha_reduce(s);
                edge_pass(s, k_update_residual, F4(0, 0, 0, 0), RED_SUM, 1);
                append_nodal(s, 0);
                beta_reduce(s);
                update_search(s);
            }
            /* switch to the nodal correction at a true-residual restart
               (src/em/mod.rs:966-990) */
            if (allow_nodal && s->control[3] == 0 && s->scalars[1].w == 0.0f && status_finite(s->scalars) &&
                (uint32_t)s->scalars[1].z >= s->nodal_after && (uint32_t)s->scalars[1].z < s->max_it) {
                s->control[3] = 1;
                restart(s);
            }
        }
        if (s->scalars[1].w != 1.0f) break;
        restart(s);
        if (s->scalars[1].w == 1.0f || (uint32_t)s->scalars[1].z >= s->max_it) break;
    }
    if (s->scalars[1].w != 1.0f && status_finite(s->scalars)) restart(s);
    memcpy(status_out, s->scalars, 32);
    if (s->scalars[1].w != 1.0f || !status_finite(s->scalars)) {
        rollback(s);
        s->can_predict = 0;
        return OEM_NOT_CONVERGED;
    }
    memcpy(s->checkpoint, s->results, (size_t)s->dims[3] * 64);
    fields(s);
    field_reduce(s);
    commit_step(s);
    memcpy(stats_out, &s->scalars[2], 64);
    for (int k = 0; k < 16; k++)
        if (!isfinite(stats_out[k])) {
            rollback(s);
            s->can_predict = 0;
            memcpy(s->results, s->checkpoint, (size_t)s->dims[3] * 64);
            return OEM_NONFINITE;
        }
    s->last_dt = initial ? 0.0 : time_s - s->time_s;
    s->can_predict = !initial && s->scalars[0].z > 0.0f;
    s->time_s = time_s;
    return OEM_OK;
}
