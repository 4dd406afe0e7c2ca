/*
 * oracle_ref.c -- FP32 restatement of the reference pressure projection.
 *
 * TEST INFRASTRUCTURE ONLY (see mhd_oracle.h).  Every function below names the
 * WGSL entry point or Rust function of the reference it restates.  Loops over
 * invocations run in workgroup order; reductions replay the reference's
 * 256-lane workgroup tree (solver.wgsl:118-120) and its 256-stride final pass
 * (solver.wgsl:199-202), so the FP32 sums are taken in the same order.
 * Built with -ffp-contract=off: no multiply-add is fused.
 */
#include "mhd_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define LANES 4
typedef struct { int32_t v[3]; } ivec3;

typedef struct {
    const oref_params *p;
    const uint32_t *mask;
    const float *occ, *phase, *oldp;
    float *velocity;  /* 4*nf: coefficient cache, then projected velocity */
    float *predicted; /* 4*nf: candidate u* */
    float *work;      /* 4*n  */
    float *partials;  /* 4*groups */
    float scalars[5][4];
    uint32_t groups;
} state;

/* ---------------------------------------------------------- periodic.wgsl:5 */
static int32_t wrap_periodic(int32_t value, uint32_t size) {
    if (value >= 0) return (int32_t)((uint32_t)value % size);
    uint32_t magnitude = (uint32_t)(-(value + 1)) + 1u;
    uint32_t remainder = magnitude % size;
    return (int32_t)(remainder == 0u ? 0u : size - remainder);
}

/* ---------------------------------------------------- solver.wgsl:17-32 */
static uint32_t idx3(ivec3 q, const uint32_t *d) {
    return (uint32_t)q.v[0] + d[0] * ((uint32_t)q.v[1] + d[1] * (uint32_t)q.v[2]);
}
static ivec3 decode3(uint32_t i, const uint32_t *d) {
    ivec3 q = {{(int32_t)(i % d[0]), (int32_t)((i / d[0]) % d[1]), (int32_t)(i / (d[0] * d[1]))}};
    return q;
}
static int periodic_axis(const state *s, uint32_t a) { return (s->p->flags[0] & (1u << a)) != 0u; }
static ivec3 wrap_cell(const state *s, ivec3 q) {
    for (uint32_t a = 0; a < 3; a++)
        if (periodic_axis(s, a)) q.v[a] = wrap_periodic(q.v[a], s->p->dims[a]);
    return q;
}
static int valid_cell(const state *s, ivec3 q) {
    for (int a = 0; a < 3; a++)
        if (q.v[a] < 0 || q.v[a] >= (int32_t)s->p->dims[a]) return 0;
    return 1;
}
static int fluid(const state *s, ivec3 pos) {
    ivec3 q = wrap_cell(s, pos);
    if (!valid_cell(s, q)) return 0;
    return s->mask[idx3(q, s->p->dims)] != 0u;
}
static int valid_face(const state *s, ivec3 q, uint32_t axis) {
    for (uint32_t a = 0; a < 3; a++) {
        int32_t lim = (int32_t)s->p->dims[a] + (a == axis ? 1 : 0);
        if (q.v[a] < 0 || q.v[a] >= lim) return 0;
    }
    return 1;
}
static int open_face(const state *s, ivec3 pos, uint32_t axis) {
    ivec3 q = wrap_cell(s, pos);
    if (!valid_face(s, q, axis)) return 0;
    ivec3 left = q;
    left.v[axis] -= 1;
    return fluid(s, left) && fluid(s, q);
}
/* face(): solver.wgsl:33-36 */
static float face_value(const state *s, ivec3 pos, uint32_t axis, int star) {
    ivec3 q = wrap_cell(s, pos);
    if (!open_face(s, q, axis)) return 0.0f;
    uint32_t i = idx3(q, s->p->faces);
    return star ? s->predicted[LANES * i + axis] : s->velocity[LANES * i + axis];
}
/* potential(): :37-39 */
static float potential(const state *s, ivec3 pos, uint32_t kind) {
    ivec3 q = wrap_cell(s, pos);
    if (!valid_cell(s, q) || !fluid(s, q)) return 0.0f;
    const float *v = s->work + LANES * idx3(q, s->p->dims);
    return kind == 0u ? v[0] : v[2];
}
/* occupancy/density/face_density: :40-42.  mix(e1,e2,t) = e1*(1-t)+e2*t. */
static float occupancy(const state *s, ivec3 pos) {
    ivec3 q = wrap_cell(s, pos);
    if (!valid_cell(s, q)) return 0.0f;
    return s->occ[idx3(q, s->p->dims)];
}
static float density(const state *s, ivec3 pos) {
    float t = occupancy(s, pos);
    return s->p->surface[1] * (1.0f - t) + s->p->physical[3] * t;
}
static float face_density(const state *s, ivec3 pos, uint32_t axis) {
    ivec3 left = pos;
    left.v[axis] -= 1;
    return 0.5f * (density(s, left) + density(s, pos));
}
/* ------------------------------------------------ interior fast paths
 * For a cell whose six neighbours all lie inside the grid no coordinate
 * wraps, so the face and neighbour records sit at fixed offsets.  The *_fast
 * helpers evaluate the same expressions as the general functions, in the
 * same order, so their results are bit-identical; they only skip the
 * per-neighbour coordinate arithmetic.  Cells on the grid's shell take the
 * general path.  Neighbour order: -x, +x, -y, +y, -z, +z. */
/* the position of cell i + 1 from that of cell i (x-fastest order) */
static void next3(ivec3 *q, const uint32_t *d) {
    if (++q->v[0] == (int32_t)d[0]) {
        q->v[0] = 0;
        if (++q->v[1] == (int32_t)d[1]) {
            q->v[1] = 0;
            q->v[2]++;
        }
    }
}
static int interior3(const uint32_t *d, ivec3 q) {
    return q.v[0] >= 1 && q.v[0] + 1 < (int32_t)d[0] && q.v[1] >= 1 && q.v[1] + 1 < (int32_t)d[1] &&
           q.v[2] >= 1 && q.v[2] + 1 < (int32_t)d[2];
}
static void cell_offsets(const uint32_t *d, int64_t co[6]) {
    const int64_t sy = d[0], sz = (int64_t)d[0] * d[1];
    co[0] = -1; co[1] = 1; co[2] = -sy; co[3] = sy; co[4] = -sz; co[5] = sz;
}
/* offset of the face record crossed towards each neighbour from the cell's
 * own (low) face record, in a grid of face records of extents f */
static void face_offsets(const uint32_t *f, int64_t fo[6]) {
    fo[0] = 0; fo[1] = 1; fo[2] = 0; fo[3] = f[0]; fo[4] = 0; fo[5] = (int64_t)f[0] * f[1];
}
/* sum over the six faces of cell i with a positive mobility beta (lane
 * `axis` of the face record) of beta * (center - neighbour value), in the
 * order -x, +x, -y, +y, -z, +z: the loop of apply (solver.wgsl:78-92) and of
 * the fine-level action (multigrid.wgsl:33-49).  The face records have
 * extents f (4 lanes each, starting at record fi); the values have stride
 * `vs` and cell extents d. */
static inline float stencil7(const float *rec, int64_t fi, const uint32_t *f, const float *val, int64_t vs,
                             uint32_t i, const uint32_t *d, float center) {
    const int64_t sy = d[0], sz = (int64_t)d[0] * d[1], fy = f[0], fz = (int64_t)f[0] * f[1];
    const int64_t ii = i;
    float out = 0.0f, beta;
    beta = rec[LANES * fi + 0];
    if (beta > 0.0f) out += beta * (center - val[vs * (ii - 1)]);
    beta = rec[LANES * (fi + 1) + 0];
    if (beta > 0.0f) out += beta * (center - val[vs * (ii + 1)]);
    beta = rec[LANES * fi + 1];
    if (beta > 0.0f) out += beta * (center - val[vs * (ii - sy)]);
    beta = rec[LANES * (fi + fy) + 1];
    if (beta > 0.0f) out += beta * (center - val[vs * (ii + sy)]);
    beta = rec[LANES * fi + 2];
    if (beta > 0.0f) out += beta * (center - val[vs * (ii - sz)]);
    beta = rec[LANES * (fi + fz) + 2];
    if (beta > 0.0f) out += beta * (center - val[vs * (ii + sz)]);
    return out;
}
static float density_at(const state *s, uint32_t i) {
    float t = s->occ[i];
    return s->p->surface[1] * (1.0f - t) + s->p->physical[3] * t;
}
/* mobility() of the face between cells iL (low side) and iR, both inside
 * the grid (the face is open). */
static float mobility_cells(const state *s, uint32_t iL, uint32_t iR) {
    const oref_params *p = s->p;
    float beta = 1.0f;
    if (p->surface[0] > 0.5f) beta = p->physical[3] / (0.5f * (density_at(s, iL) + density_at(s, iR)));
    if (p->flags[3] == 0u) return beta;
    if (s->mask[iR] == 0u || s->mask[iL] == 0u) return 0.0f;
    float f = fminf(s->phase[iR], s->phase[iL]);
    float drag = p->solve[3] * (1.0f - f) * (1.0f - f) / (f * f * f + 1e-3f);
    return beta / (1.0f + p->physical[1] * drag);
}

/* mobility(): :43-51 */
static float mobility(const state *s, ivec3 pos, uint32_t axis) {
    const oref_params *p = s->p;
    float beta = 1.0f;
    ivec3 left = pos;
    left.v[axis] -= 1;
    if (p->surface[0] > 0.5f) beta = p->physical[3] / face_density(s, pos, axis);
    if (p->flags[3] == 0u) return beta;
    if (!fluid(s, pos) || !fluid(s, left)) return 0.0f;
    float fa = s->phase[idx3(wrap_cell(s, pos), p->dims)];
    float fb = s->phase[idx3(wrap_cell(s, left), p->dims)];
    float f = fminf(fa, fb);
    float drag = p->solve[3] * (1.0f - f) * (1.0f - f) / (f * f * f + 1e-3f);
    return beta / (1.0f + p->physical[1] * drag);
}
static int mean_free_pressure(const state *s) { return s->p->initial[3] > 0.0f; }
static int pinned_anchor(const state *s, uint32_t i) {
    return !mean_free_pressure(s) && (s->mask[i] & 3u) == 2u;
}
/* diagonal(): :60-64 */
static float diagonal(const state *s, ivec3 pos) {
    float d = 0.0f;
    if (interior3(s->p->dims, pos)) {
        const uint32_t i = idx3(pos, s->p->dims);
        int64_t co[6];
        cell_offsets(s->p->dims, co);
        for (int t = 0; t < 6; t++) {
            const uint32_t j = (uint32_t)((int64_t)i + co[t]);
            if (s->mask[j] != 0u) d += (t & 1) ? mobility_cells(s, i, j) : mobility_cells(s, j, i);
        }
        if (pinned_anchor(s, i)) return 1.0f;
        return fmaxf(d, 1e-30f);
    }
    for (uint32_t axis = 0; axis < 3; axis++)
        for (int sign = -1; sign <= 1; sign += 2) {
            ivec3 q = pos;
            q.v[axis] += sign;
            if (fluid(s, q)) {
                ivec3 fp = pos;
                if (sign > 0) fp.v[axis] += 1;
                d += mobility(s, fp, axis);
            }
        }
    if (pinned_anchor(s, idx3(pos, s->p->dims))) return 1.0f;
    return fmaxf(d, 1e-30f);
}
/* laplacian(): :65-69 */
static float laplacian(const state *s, ivec3 pos, uint32_t kind) {
    if (interior3(s->p->dims, pos)) {
        const uint32_t i = idx3(pos, s->p->dims), k = kind == 0u ? 0u : 2u;
        const float *w = s->work;
        const float center = s->mask[i] != 0u ? w[LANES * i + k] : 0.0f;
        float out = 0.0f;
        int64_t co[6];
        cell_offsets(s->p->dims, co);
        for (int t = 0; t < 6; t++) {
            const uint32_t j = (uint32_t)((int64_t)i + co[t]);
            if (s->mask[j] != 0u) {
                const float beta = (t & 1) ? mobility_cells(s, i, j) : mobility_cells(s, j, i);
                out += beta * (center - w[LANES * j + k]);
            }
        }
        return out;
    }
    float center = potential(s, pos, kind), out = 0.0f;
    for (uint32_t axis = 0; axis < 3; axis++)
        for (int sign = -1; sign <= 1; sign += 2) {
            ivec3 q = pos;
            q.v[axis] += sign;
            if (fluid(s, q)) {
                ivec3 fp = pos;
                if (sign > 0) fp.v[axis] += 1;
                out += mobility(s, fp, axis) * (center - potential(s, q, kind));
            }
        }
    return out;
}
/* cached_mobility/cached_diagonal/apply(): :74-92 */
static float cached_mobility(const state *s, ivec3 pos, uint32_t axis) {
    return s->velocity[LANES * idx3(wrap_cell(s, pos), s->p->faces) + axis];
}
static float cached_diagonal(const state *s, uint32_t i) { return s->velocity[LANES * i + 3]; }
static float apply_cached(const state *s, ivec3 pos, uint32_t kind) {
    if (pinned_anchor(s, idx3(pos, s->p->dims))) return potential(s, pos, kind);
    if (interior3(s->p->dims, pos) && s->mask[idx3(pos, s->p->dims)] != 0u) {
        const uint32_t i = idx3(pos, s->p->dims), k = kind == 1u ? 2u : 0u;
        const int64_t fi = idx3(pos, s->p->faces);
        const float *c = s->velocity, *w = s->work;
        return stencil7(c, fi, s->p->faces, w + k, LANES, i, s->p->dims, w[LANES * i + k]);
    }
    float center = potential(s, pos, kind), out = 0.0f;
    for (uint32_t axis = 0; axis < 3; axis++)
        for (int sign = -1; sign <= 1; sign += 2) {
            ivec3 fp = pos;
            if (sign > 0) fp.v[axis] += 1;
            float beta = cached_mobility(s, fp, axis);
            if (beta > 0.0f) {
                ivec3 q = pos;
                q.v[axis] += sign;
                const float *v = s->work + LANES * idx3(wrap_cell(s, q), s->p->dims);
                out += beta * (center - (kind == 1u ? v[2] : v[0]));
            }
        }
    return out;
}
/* divergence()/rhs(): :104-107 */
static float divergence(const state *s, ivec3 pos, int star) {
    float sum = 0.0f;
    if (interior3(s->p->dims, pos)) {
        const uint32_t i = idx3(pos, s->p->dims);
        const int64_t fi = idx3(pos, s->p->faces);
        const float *f = star ? s->predicted : s->velocity;
        int64_t co[6], fo[6];
        cell_offsets(s->p->dims, co);
        face_offsets(s->p->faces, fo);
        const int ci = s->mask[i] != 0u;
        for (uint32_t a = 0; a < 3; a++) {
            const int lo = ci && s->mask[(int64_t)i + co[2 * a]] != 0u;
            const int hi = ci && s->mask[(int64_t)i + co[2 * a + 1]] != 0u;
            const float fh = hi ? f[LANES * (fi + fo[2 * a + 1]) + a] : 0.0f;
            const float fl = lo ? f[LANES * fi + a] : 0.0f;
            sum += fh - fl;
        }
        return sum / s->p->physical[0];
    }
    for (uint32_t axis = 0; axis < 3; axis++) {
        ivec3 q = pos;
        q.v[axis] += 1;
        sum += face_value(s, q, axis, star) - face_value(s, pos, axis, star);
    }
    return sum / s->p->physical[0];
}
static float rhs(const state *s, ivec3 pos) {
    if (pinned_anchor(s, idx3(pos, s->p->dims))) return 0.0f;
    return -s->p->physical[0] * s->p->physical[0] * divergence(s, pos, 1);
}
/* old_potential(): :164-167 */
static float old_potential(const state *s, ivec3 pos) {
    ivec3 q = wrap_cell(s, pos);
    if (!fluid(s, q)) return 0.0f;
    uint32_t i = idx3(q, s->p->dims), anchor = s->mask[i] >> 2u;
    return (s->oldp[i] - s->oldp[anchor]) * s->p->physical[1] / s->p->physical[3];
}

/* ------------------------------------------------ workgroup reductions */
static void tree256(float red[256][4]) {
    for (uint32_t stride = 128u; stride > 0u; stride /= 2u)
        for (uint32_t l = 0; l < stride; l++)
            for (int c = 0; c < 4; c++) red[l][c] += red[l + stride][c];
}
/* The 1-workgroup second stage (initial_reduce, :199-203 and the others). */
static void reduce_partials(const state *s, float total[4]) {
    float red[256][4];
    for (uint32_t l = 0; l < 256u; l++) {
        float sum[4] = {0, 0, 0, 0};
        for (uint32_t i = l; i < s->groups; i += 256u)
            for (int c = 0; c < 4; c++) sum[c] += s->partials[LANES * i + c];
        memcpy(red[l], sum, sizeof sum);
    }
    tree256(red);
    memcpy(total, red[0], 4 * sizeof(float));
}
static int converged_flag(const state *s) { return s->scalars[1][2] >= 0.5f; }

/* ------------------------------------------------------------- kernels */
/* pressure_coefficients: :93-103 */
static void k_pressure_coefficients(state *s) {
    const oref_params *p = s->p;
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)p->faces[3]; ii++) {
        uint32_t i = (uint32_t)ii;
        ivec3 pos = decode3(i, p->faces);
        float coeff[4] = {0, 0, 0, 0};
        if (interior3(p->dims, pos)) {
            const uint32_t c = idx3(pos, p->dims);
            int64_t co[6];
            cell_offsets(p->dims, co);
            for (uint32_t axis = 0; axis < 3; axis++) {
                const uint32_t l = (uint32_t)((int64_t)c + co[2 * axis]);
                if (s->mask[l] != 0u && s->mask[c] != 0u) coeff[axis] = mobility_cells(s, l, c);
            }
        } else {
            for (uint32_t axis = 0; axis < 3; axis++)
                if (open_face(s, pos, axis)) coeff[axis] = mobility(s, pos, axis);
        }
        if (i < p->dims[3] && s->mask[i] != 0u) coeff[3] = diagonal(s, decode3(i, p->dims));
        memcpy(s->velocity + LANES * i, coeff, sizeof coeff);
    }
}
/* pressure_warm: :170-176 */
static void k_pressure_warm(state *s) {
    const oref_params *p = s->p;
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)p->faces[3]; ii++) {
        uint32_t i = (uint32_t)ii;
        ivec3 pos = decode3(i, p->faces);
        float *out = s->predicted + LANES * i;
        for (uint32_t axis = 0; axis < 3; axis++)
            if (open_face(s, pos, axis)) {
                ivec3 left = pos;
                left.v[axis] -= 1;
                out[axis] -= mobility(s, pos, axis) * (old_potential(s, pos) - old_potential(s, left)) /
                             p->physical[0];
            }
    }
}
/* pressure_guess: :177-180 */
static void k_pressure_guess(state *s) {
    memset(s->work, 0, sizeof(float) * LANES * s->p->dims[3]);
    s->scalars[1][3] = 0.0f;
    s->scalars[2][0] = mean_free_pressure(s) ? 1.0f : 0.0f;
}
/* pressure_commit: :181-184 */
static void k_pressure_commit(state *s) {
    const oref_params *p = s->p;
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)p->dims[3]; ii++) {
        uint32_t i = (uint32_t)ii;
        if (s->mask[i] != 0u) s->work[LANES * i] += old_potential(s, decode3(i, p->dims));
    }
}
/* pressure_refresh: :185-197 */
static void k_pressure_refresh(state *s) {
    const oref_params *p = s->p;
    const int mf = mean_free_pressure(s);
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < (int64_t)s->groups; g++) {
        float red[256][4];
        ivec3 pos = decode3((uint32_t)g * 256u, p->dims);
        for (uint32_t l = 0; l < 256u; l++, next3(&pos, p->dims)) {
            uint32_t i = (uint32_t)g * 256u + l;
            float sum[4] = {0, 0, 0, 0};
            if (i < p->dims[3] && s->mask[i] != 0u) {
                float b = rhs(s, pos), r = b - apply_cached(s, pos, 0u), d = cached_diagonal(s, i);
                s->work[LANES * i + 1] = r;
                s->work[LANES * i + 2] = r / d;
                float physical = -p->physical[0] * p->physical[0] * divergence(s, pos, 1);
                float true_residual = physical - laplacian(s, pos, 0u);
                sum[0] = r * r / d;
                sum[1] = true_residual * true_residual;
                sum[2] = physical * physical;
                sum[3] = mf ? r : 0.0f;
            }
            memcpy(red[l], sum, sizeof sum);
        }
        tree256(red);
        memcpy(s->partials + LANES * g, red[0], 4 * sizeof(float));
    }
}
/* initial_reduce: :198-203 */
static void k_initial_reduce(state *s) {
    float total[4];
    reduce_partials(s, total);
    memcpy(s->scalars[0], total, sizeof total);
    float flag = (total[1] <= s->p->solve[0] * total[2] + s->p->solve[1] || total[2] == 0.0f) ? 1.0f : 0.0f;
    float w = s->scalars[1][3];
    s->scalars[1][0] = 0.0f;
    s->scalars[1][1] = 0.0f;
    s->scalars[1][2] = flag;
    s->scalars[1][3] = w;
}
/* pressure_apply: :204-210 */
static void k_pressure_apply(state *s) {
    const oref_params *p = s->p;
    const int conv = converged_flag(s);
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < (int64_t)s->groups; g++) {
        float red[256][4];
        ivec3 pos = decode3((uint32_t)g * 256u, p->dims);
        for (uint32_t l = 0; l < 256u; l++, next3(&pos, p->dims)) {
            uint32_t i = (uint32_t)g * 256u + l;
            float value = 0.0f;
            if (i < p->dims[3] && s->mask[i] != 0u && !conv) {
                float a = apply_cached(s, pos, 1u);
                s->work[LANES * i + 3] = a;
                value = s->work[LANES * i + 2] * a;
            }
            red[l][0] = value;
            red[l][1] = red[l][2] = red[l][3] = 0.0f;
        }
        tree256(red);
        memcpy(s->partials + LANES * g, red[0], 4 * sizeof(float));
    }
}
/* alpha_reduce: :211-215 */
static void k_alpha_reduce(state *s) {
    float total[4];
    reduce_partials(s, total);
    float alpha = 0.0f;
    if (!converged_flag(s)) alpha = s->scalars[0][0] / fmaxf(total[0], 1e-35f);
    s->scalars[1][0] = alpha;
}
/* update: :216-230 */
static void k_update(state *s) {
    const oref_params *p = s->p;
    const int conv = converged_flag(s), mf = mean_free_pressure(s);
    const float a = s->scalars[1][0];
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < (int64_t)s->groups; g++) {
        float red[256][4];
        for (uint32_t l = 0; l < 256u; l++) {
            uint32_t i = (uint32_t)g * 256u + l;
            float sum[4] = {0, 0, 0, 0};
            if (i < p->dims[3] && s->mask[i] != 0u && !conv) {
                float *w = s->work + LANES * i;
                float v[4] = {w[0], w[1], w[2], w[3]};
                float r = v[1] - a * v[3];
                float diag = cached_diagonal(s, i);
                if (mf) {
                    w[0] = v[0] + a * (v[2] - s->work[LANES * (s->mask[i] >> 2u) + 2]);
                    w[1] = r;
                    w[3] = diag;
                } else {
                    w[0] = v[0] + a * v[2];
                    w[1] = r;
                    w[2] = v[2];
                    w[3] = diag;
                }
                sum[0] = r * r / diag;
                sum[1] = r * r;
                sum[3] = mf ? r : 0.0f;
            }
            memcpy(red[l], sum, sizeof sum);
        }
        tree256(red);
        memcpy(s->partials + LANES * g, red[0], 4 * sizeof(float));
    }
}
/* beta_reduce: :231-239 */
static void k_beta_reduce(state *s) {
    float total[4];
    reduce_partials(s, total);
    if (!converged_flag(s)) {
        const oref_params *p = s->p;
        s->scalars[1][3] += 1.0f;
        s->scalars[1][1] = total[0] / fmaxf(s->scalars[0][0], 1e-35f);
        s->scalars[0][0] = total[0];
        s->scalars[0][1] = total[1];
        s->scalars[1][2] = total[1] <= (p->solve[0] * s->scalars[0][2] + p->solve[1]) / p->solve[2] ? 1.0f : 0.0f;
    }
}
/* search: :240-244 */
static void k_search(state *s) {
    const oref_params *p = s->p;
    if (converged_flag(s)) return;
    const float beta = s->scalars[1][1];
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)p->dims[3]; ii++) {
        uint32_t i = (uint32_t)ii;
        if (s->mask[i] == 0u) continue;
        float *w = s->work + LANES * i;
        w[2] = w[1] / w[3] + beta * w[2];
    }
}
/* pressure_residual_mean: pressure_subspace.wgsl:3-7 */
static void k_pressure_residual_mean(state *s) {
    float red[256][4];
    for (uint32_t l = 0; l < 256u; l++) {
        float sum = 0.0f;
        for (uint32_t i = l; i < s->groups; i += 256u) sum += s->partials[LANES * i + 3];
        red[l][0] = sum;
        red[l][1] = red[l][2] = red[l][3] = 0.0f;
    }
    tree256(red);
    s->scalars[2][1] = red[0][0] * s->p->initial[3];
}
/* project_pressure_residual: pressure_subspace.wgsl:8-20 */
static void k_project_pressure_residual(state *s, int initial) {
    const oref_params *p = s->p;
    const int conv = converged_flag(s);
    const float mean = s->scalars[2][1];
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < (int64_t)s->groups; g++) {
        float red[256][4];
        for (uint32_t l = 0; l < 256u; l++) {
            uint32_t i = (uint32_t)g * 256u + l;
            float value[4] = {0, 0, 0, 0};
            if (i < p->dims[3] && s->mask[i] != 0u && (initial || !conv)) {
                float *w = s->work + LANES * i;
                float r = w[1] - mean, d = cached_diagonal(s, i);
                w[1] = r;
                if (initial) w[2] = r / d;
                value[0] = r * r / d;
                value[1] = r * r;
            }
            memcpy(red[l], value, sizeof value);
        }
        tree256(red);
        float *old = s->partials + LANES * g;
        float nv[4] = {red[0][0], initial ? old[1] : red[0][1], old[2], 0.0f};
        memcpy(old, nv, sizeof nv);
    }
}
/* pressure_check / check_reduce: :317-328 */
static void k_pressure_check(state *s) {
    const oref_params *p = s->p;
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < (int64_t)s->groups; g++) {
        float red[256][4];
        ivec3 pos = decode3((uint32_t)g * 256u, p->dims);
        for (uint32_t l = 0; l < 256u; l++, next3(&pos, p->dims)) {
            uint32_t i = (uint32_t)g * 256u + l;
            red[l][0] = red[l][1] = red[l][2] = red[l][3] = 0.0f;
            if (i < p->dims[3] && s->mask[i] != 0u) {
                float b = -p->physical[0] * p->physical[0] * divergence(s, pos, 1);
                float r = b - laplacian(s, pos, 0u);
                red[l][1] = r * r;
            }
        }
        tree256(red);
        memcpy(s->partials + LANES * g, red[0], 4 * sizeof(float));
    }
}
static void k_check_reduce(state *s) {
    float total[4];
    reduce_partials(s, total);
    s->scalars[0][1] = total[1];
    s->scalars[1][2] = total[1] <= s->p->solve[0] * s->scalars[0][2] + s->p->solve[1] ? 1.0f : 0.0f;
}
/* correct: :245-250 */
static void k_correct(state *s) {
    const oref_params *p = s->p;
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)p->faces[3]; ii++) {
        uint32_t i = (uint32_t)ii;
        ivec3 pos = decode3(i, p->faces);
        float out[4] = {0, 0, 0, 0};
        if (interior3(p->dims, pos)) {
            const uint32_t c = idx3(pos, p->dims);
            int64_t co[6];
            cell_offsets(p->dims, co);
            for (uint32_t axis = 0; axis < 3; axis++) {
                const uint32_t l = (uint32_t)((int64_t)c + co[2 * axis]);
                if (s->mask[l] != 0u && s->mask[c] != 0u)
                    out[axis] = s->predicted[LANES * i + axis] -
                                mobility_cells(s, l, c) * (s->work[LANES * c] - s->work[LANES * l]) / p->physical[0];
            }
        } else {
            for (uint32_t axis = 0; axis < 3; axis++)
                if (open_face(s, pos, axis)) {
                    ivec3 left = pos;
                    left.v[axis] -= 1;
                    out[axis] = face_value(s, pos, axis, 1) -
                                mobility(s, pos, axis) * (potential(s, pos, 0u) - potential(s, left, 0u)) /
                                    p->physical[0];
                }
        }
        /* Each invocation writes only its own face record; the cache it
           reads (mobility is uncached here) is not used any more. */
        memcpy(s->velocity + LANES * i, out, sizeof out);
    }
}

/* ------------------------------------------ multigrid (multigrid.wgsl) */
typedef struct { uint32_t dims[4], child[4], faces[4], location[4]; } level_t;

struct oref_mg {
    const oref_params *p;
    const uint32_t *mask;
    const float *cache; /* the fine coefficient cache (velocity buffer) */
    float *work, *temp;  /* fine work vec4[n]; temp = predicted.w lane */
    float *coeff, *value;
    level_t *levels;
    uint32_t nlevels;
    uint64_t coarse_cells;
    int meanfree;
    const state *fluid_state; /* converged flag / beta source; NULL in probes */
    float *partials;
    uint32_t groups;
};

static int mg_converged(const struct oref_mg *mg) {
    return mg->fluid_state ? converged_flag(mg->fluid_state) : 0;
}
static ivec3 mg_canonical(const struct oref_mg *mg, const level_t *L, ivec3 q, const uint32_t *d) {
    (void)mg;
    for (uint32_t a = 0; a < 3; a++)
        if (L->location[3] & (1u << a)) q.v[a] = wrap_periodic(q.v[a], d[a]);
    return q;
}
static int mg_valid(ivec3 q, const uint32_t *d) {
    for (int a = 0; a < 3; a++)
        if (q.v[a] < 0 || q.v[a] >= (int32_t)d[a]) return 0;
    return 1;
}
static int fine_active(const struct oref_mg *mg, uint32_t i) {
    return mg->mask[i] != 0u && (mg->meanfree || (mg->mask[i] & 3u) == 1u);
}
/* edge(): multigrid.wgsl:24-28 */
static float mg_edge(const struct oref_mg *mg, const level_t *L, ivec3 q, uint32_t axis, int sign,
                     const uint32_t *d, uint32_t offset, int fine) {
    ivec3 f = q;
    if (sign > 0) f.v[axis] += 1;
    f = mg_canonical(mg, L, f, d);
    if (fine) return mg->cache[LANES * idx3(f, L->faces) + axis];
    return mg->coeff[LANES * (offset + idx3(f, d)) + axis];
}
/* solution(): :29-32 */
static float mg_solution(const struct oref_mg *mg, uint32_t i, uint32_t offset, int fine, int temp) {
    if (fine) return temp ? mg->temp[i] : mg->work[LANES * i + 3];
    const float *v = mg->value + LANES * (offset + i);
    return temp ? v[2] : v[1];
}
/* action(): :33-49 */
static float mg_action(const struct oref_mg *mg, const level_t *L, ivec3 q, const uint32_t *d,
                       uint32_t offset, int fine, int temp) {
    uint32_t i = idx3(q, d);
    if (fine && interior3(d, q)) {
        /* interior fast path (same operations, same order as below) */
        const float *src = temp ? mg->temp : mg->work + 3;
        const int64_t vs = temp ? 1 : LANES;
        return stencil7(mg->cache, idx3(q, L->faces), L->faces, src, vs, i, d, src[vs * i]);
    }
    float center = mg_solution(mg, i, offset, fine, temp), out = 0.0f;
    if (interior3(d, q)) {
        int64_t co[6];
        cell_offsets(d, co);
        out = mg->coeff[LANES * (offset + i) + 3] * center;
        const uint32_t lane = temp ? 2u : 1u;
        for (int t = 0; t < 6; t++) {
            const int64_t f = (t & 1) ? (int64_t)i + co[t] : (int64_t)i;
            const float beta = mg->coeff[LANES * (offset + f) + (t >> 1)];
            if (beta > 0.0f) out += beta * (center - mg->value[LANES * (offset + (int64_t)i + co[t]) + lane]);
        }
        return out;
    }
    if (fine) {
        for (uint32_t a = 0; a < 3; a++)
            for (int s = -1; s <= 1; s += 2) {
                float beta = mg_edge(mg, L, q, a, s, d, offset, 1);
                if (beta > 0.0f) {
                    ivec3 n = q;
                    n.v[a] += s;
                    n = mg_canonical(mg, L, n, d);
                    out += beta * (center - mg_solution(mg, idx3(n, d), offset, 1, temp));
                }
            }
        return out;
    }
    out = mg->coeff[LANES * (offset + i) + 3] * center;
    for (uint32_t a = 0; a < 3; a++)
        for (int s = -1; s <= 1; s += 2) {
            ivec3 n = q;
            n.v[a] += s;
            n = mg_canonical(mg, L, n, d);
            if (!mg_valid(n, d)) continue;
            float beta = mg_edge(mg, L, q, a, s, d, offset, 0);
            if (beta > 0.0f) out += beta * (center - mg_solution(mg, idx3(n, d), offset, 0, temp));
        }
    return out;
}
/* build(): :50-65 */
static void mg_build_level(struct oref_mg *mg, const level_t *L) {
    const int fine = L->location[2] == 1u;
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)L->dims[3]; ii++) {
        uint32_t i = (uint32_t)ii;
        ivec3 q = decode3(i, L->dims);
        float c[4] = {0, 0, 0, 0}, diag = 0.0f;
        for (int z = 0; z < 2; z++)
            for (int y = 0; y < 2; y++)
                for (int x = 0; x < 2; x++) {
                    ivec3 child = {{2 * q.v[0] + x, 2 * q.v[1] + y, 2 * q.v[2] + z}};
                    if (!mg_valid(child, L->child)) continue;
                    uint32_t ci = idx3(child, L->child);
                    if (fine) {
                        if (!fine_active(mg, ci)) continue;
                    } else {
                        float gamma = mg->coeff[LANES * (L->location[1] + ci) + 3];
                        c[3] += gamma;
                        diag += gamma;
                    }
                    for (uint32_t a = 0; a < 3; a++)
                        for (int s = -1; s <= 1; s += 2) {
                            ivec3 n = child;
                            n.v[a] += s;
                            n = mg_canonical(mg, L, n, L->child);
                            if (!mg_valid(n, L->child)) continue;
                            float beta = mg_edge(mg, L, child, a, s, L->child, L->location[1], fine);
                            if (beta == 0.0f) continue;
                            if (fine && !mg->meanfree && (mg->mask[idx3(n, L->child)] & 3u) == 2u) {
                                c[3] += beta;
                                diag += beta;
                                continue;
                            }
                            ivec3 parent = {{n.v[0] / 2, n.v[1] / 2, n.v[2] / 2}};
                            if (parent.v[0] == q.v[0] && parent.v[1] == q.v[1] && parent.v[2] == q.v[2]) continue;
                            diag += beta;
                            if (s < 0) c[a] += beta;
                        }
                }
        memcpy(mg->coeff + LANES * (L->location[0] + i), c, sizeof c);
        float v[4] = {0, 0, 0, diag};
        memcpy(mg->value + LANES * (L->location[0] + i), v, sizeof v);
    }
}
/* jacobi_step(): :66-71 (temp=false is smooth_to_temp) */
static void mg_jacobi(struct oref_mg *mg, const level_t *L, int temp) {
    if (mg_converged(mg)) return;
    const int fine = L->location[2] == 0u;
    const uint32_t off = L->location[0];
#pragma omp parallel for schedule(static)
    for (int64_t row = 0; row < (int64_t)L->dims[1] * L->dims[2]; row++)
    for (uint32_t x = 0; x < L->dims[0]; x++) {
        uint32_t i = x + L->dims[0] * (uint32_t)row;
        ivec3 q = {{(int32_t)x, (int32_t)(row % L->dims[1]), (int32_t)(row / L->dims[1])}};
        float d, r;
        if (fine) {
            d = mg->cache[LANES * i + 3];
            r = mg->work[LANES * i + 1];
            if (!fine_active(mg, i)) d = 0.0f;
        } else {
            d = mg->value[LANES * (off + i) + 3];
            r = mg->value[LANES * (off + i) + 0];
        }
        float next = 0.0f;
        if (d > 0.0f)
            next = mg_solution(mg, i, off, fine, temp) +
                   (2.0f / 3.0f) * (r - mg_action(mg, L, q, L->dims, off, fine, temp)) / d;
        if (fine) {
            if (temp) mg->work[LANES * i + 3] = next;
            else mg->temp[i] = next;
        } else {
            if (temp) mg->value[LANES * (off + i) + 1] = next;
            else mg->value[LANES * (off + i) + 2] = next;
        }
    }
}
/* restrict_residual(): :74-83 */
static void mg_restrict(struct oref_mg *mg, const level_t *L) {
    if (mg_converged(mg)) return;
    const int fine = L->location[2] == 1u;
#pragma omp parallel for schedule(static)
    for (int64_t row = 0; row < (int64_t)L->dims[1] * L->dims[2]; row++)
    for (uint32_t x = 0; x < L->dims[0]; x++) {
        uint32_t i = x + L->dims[0] * (uint32_t)row;
        ivec3 q = {{(int32_t)x, (int32_t)(row % L->dims[1]), (int32_t)(row / L->dims[1])}};
        float sum = 0.0f;
        for (int z = 0; z < 2; z++)
            for (int y = 0; y < 2; y++)
                for (int x = 0; x < 2; x++) {
                    ivec3 child = {{2 * q.v[0] + x, 2 * q.v[1] + y, 2 * q.v[2] + z}};
                    if (!mg_valid(child, L->child)) continue;
                    uint32_t ci = idx3(child, L->child);
                    float r;
                    if (fine) {
                        if (!fine_active(mg, ci)) continue;
                        r = mg->work[LANES * ci + 1];
                    } else {
                        r = mg->value[LANES * (L->location[1] + ci)];
                    }
                    sum += r - mg_action(mg, L, child, L->child, L->location[1], fine, 0);
                }
        float *v = mg->value + LANES * (L->location[0] + i);
        v[0] = sum;
        v[1] = 0.0f;
        v[2] = 0.0f;
    }
}
/* prolong(): :84-88 */
static void mg_prolong(struct oref_mg *mg, const level_t *L) {
    if (mg_converged(mg)) return;
#pragma omp parallel for schedule(static)
    for (int64_t row = 0; row < (int64_t)L->child[1] * L->child[2]; row++)
    for (uint32_t x = 0; x < L->child[0]; x++) {
        uint32_t i = x + L->child[0] * (uint32_t)row;
        ivec3 q = {{(int32_t)x, (int32_t)(row % L->child[1]), (int32_t)(row / L->child[1])}};
        ivec3 par = {{q.v[0] / 2, q.v[1] / 2, q.v[2] / 2}};
        float correction = mg->value[LANES * (L->location[0] + idx3(par, L->dims)) + 1];
        if (L->location[2] == 1u) {
            if (fine_active(mg, i)) mg->work[LANES * i + 3] += correction;
        } else {
            mg->value[LANES * (L->location[1] + i) + 1] += correction;
        }
    }
}
/* coarse_solve(): :106-131, COARSE_SWEEPS = 8 (multigrid.rs:3) */
#define COARSE_SWEEPS 8u
void mg_coarse_solve_level(struct oref_mg *mg, const level_t *L) {
    if (mg_converged(mg)) return;
    const int fine = L->location[2] == 0u;
    const uint32_t off = L->location[0];
    float sol[256], next[256], rhsv[256], diagv[256], reaction[256];
    ivec3 qv[256];
    for (uint32_t i = 0; i < 256u; i++) {
        rhsv[i] = diagv[i] = reaction[i] = 0.0f;
        qv[i].v[0] = qv[i].v[1] = qv[i].v[2] = 0;
        if (i < L->dims[3]) {
            qv[i] = decode3(i, L->dims);
            if (fine) {
                if (fine_active(mg, i)) {
                    rhsv[i] = mg->work[LANES * i + 1];
                    diagv[i] = mg->cache[LANES * i + 3];
                }
            } else {
                rhsv[i] = mg->value[LANES * (off + i)];
                diagv[i] = mg->value[LANES * (off + i) + 3];
                reaction[i] = mg->coeff[LANES * (off + i) + 3];
            }
        }
        sol[i] = 0.0f;
    }
    for (uint32_t step = 0; step < COARSE_SWEEPS; step++) {
        for (uint32_t i = 0; i < 256u; i++) {
            float center = sol[i], nx = 0.0f;
            if (i < L->dims[3] && diagv[i] > 0.0f) {
                float a = reaction[i] * center;
                for (uint32_t axis = 0; axis < 3; axis++)
                    for (int s = -1; s <= 1; s += 2) {
                        ivec3 n = qv[i];
                        n.v[axis] += s;
                        n = mg_canonical(mg, L, n, L->dims);
                        if (!mg_valid(n, L->dims)) continue;
                        uint32_t ni = idx3(n, L->dims);
                        float neighbor = sol[ni];
                        if (fine && !fine_active(mg, ni)) neighbor = 0.0f;
                        a += mg_edge(mg, L, qv[i], axis, s, L->dims, off, fine) * (center - neighbor);
                    }
                nx = center + (2.0f / 3.0f) * (rhsv[i] - a) / diagv[i];
            }
            next[i] = nx;
        }
        memcpy(sol, next, sizeof sol);
    }
    for (uint32_t i = 0; i < L->dims[3]; i++) {
        if (fine) mg->work[LANES * i + 3] = sol[i];
        else mg->value[LANES * (off + i) + 1] = sol[i];
    }
}
/* diagonal_start(): :133-139 */
static void mg_diagonal_start(struct oref_mg *mg, const level_t *L) {
    if (mg_converged(mg)) return;
    const uint32_t off = L->location[0];
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)L->dims[3]; ii++) {
        uint32_t i = (uint32_t)ii;
        float z = 0.0f;
        if (L->location[2] == 0u) {
            if (fine_active(mg, i)) z = (2.0f / 3.0f) * mg->work[LANES * i + 1] / mg->cache[LANES * i + 3];
            mg->work[LANES * i + 3] = z;
        } else {
            float *v = mg->value + LANES * (off + i);
            if (v[3] > 0.0f) z = (2.0f / 3.0f) * v[0] / v[3];
            v[1] = z;
        }
    }
}
/* commit_smooth(): :140-144 */
static void mg_commit(struct oref_mg *mg, const level_t *L) {
    if (mg_converged(mg)) return;
    const uint32_t off = L->location[0];
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)L->dims[3]; ii++) {
        const uint32_t i = (uint32_t)ii;
        if (L->location[2] == 0u) mg->work[LANES * i + 3] = mg->temp[i];
        else mg->value[LANES * (off + i) + 1] = mg->value[LANES * (off + i) + 2];
    }
}
/* cycle_stages(): multigrid.rs:67-82, executed in order. */
static void mg_cycle(struct oref_mg *mg) {
    uint32_t L = mg->nlevels;
    for (uint32_t l = 0; l + 1 < L; l++) {
        mg_diagonal_start(mg, &mg->levels[l]);
        mg_restrict(mg, &mg->levels[l + 1]);
    }
    mg_coarse_solve_level(mg, &mg->levels[L - 1]);
    for (int32_t l = (int32_t)L - 2; l >= 0; l--) {
        mg_prolong(mg, &mg->levels[l + 1]);
        mg_jacobi(mg, &mg->levels[l], 0);
        mg_commit(mg, &mg->levels[l]);
    }
}
/* dot_partial(): :90-96 */
static void mg_dot_partial(struct oref_mg *mg, int initial) {
    const level_t *L = &mg->levels[0];
    const int conv = mg_converged(mg);
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < (int64_t)mg->groups; g++) {
        float red[256][4];
        for (uint32_t l = 0; l < 256u; l++) {
            uint32_t i = (uint32_t)g * 256u + l;
            float v = 0.0f;
            if (i < L->dims[3] && fine_active(mg, i) && !conv) {
                v = mg->work[LANES * i + 1] * mg->work[LANES * i + 3];
                if (initial) mg->work[LANES * i + 2] = mg->work[LANES * i + 3];
            }
            red[l][0] = v;
            red[l][1] = red[l][2] = red[l][3] = 0.0f;
        }
        tree256(red);
        if (!conv) mg->partials[LANES * g] = red[0][0];
    }
}
/* preconditioned_search(): :101-102 */
static void mg_preconditioned_search(struct oref_mg *mg) {
    if (mg_converged(mg)) return;
    const float beta = mg->fluid_state->scalars[1][1];
    const level_t *L = &mg->levels[0];
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)L->dims[3]; ii++) {
        uint32_t i = (uint32_t)ii;
        if (!fine_active(mg, i)) continue;
        float *w = mg->work + LANES * i;
        w[2] = w[3] + beta * w[2];
    }
}

/* hierarchy(): multigrid.rs:25-65 */
int oref_hierarchy(const uint32_t dims[4], uint32_t *nlevels, uint64_t *coarse_cells,
                   uint32_t *level_dims, uint32_t max_levels) {
    uint64_t count = 1;
    for (int a = 0; a < 3; a++)
        if (__builtin_mul_overflow(count, (uint64_t)dims[a], &count)) return 1; /* "grid count overflow" */
    for (int a = 0; a < 3; a++)
        if (dims[a] > 0x7FFFFFFFu) return 2; /* "exceed signed shader coordinates" */
    if (dims[0] == 0 || dims[1] == 0 || dims[2] == 0 || count != (uint64_t)dims[3]) return 3;
    uint32_t d[3] = {dims[0], dims[1], dims[2]}, n = 1;
    uint64_t offset = 0;
    if (level_dims && max_levels > 0) {
        level_dims[0] = d[0]; level_dims[1] = d[1]; level_dims[2] = d[2]; level_dims[3] = dims[3];
    }
    while (d[0] > 4 || d[1] > 4 || d[2] > 4) {
        for (int a = 0; a < 3; a++) d[a] = (d[a] + 1) / 2;
        uint64_t c = (uint64_t)d[0] * d[1] * d[2];
        if (offset > 0xFFFFFFFFull) return 4; /* u32::try_from(offset) */
        if (level_dims && n < max_levels) {
            level_dims[4 * n] = d[0]; level_dims[4 * n + 1] = d[1];
            level_dims[4 * n + 2] = d[2]; level_dims[4 * n + 3] = (uint32_t)c;
        }
        offset += c;
        n++;
        if (offset > 0xFFFFFFFFull) return 4; /* "Coarse pressure indices exceed u32" */
    }
    *nlevels = n;
    *coarse_cells = offset;
    return 0;
}

static struct oref_mg *mg_new(const oref_params *p, const uint32_t *mask, const float *cache, float *work,
                              int meanfree) {
    uint32_t nl;
    uint64_t cc;
    if (oref_hierarchy(p->dims, &nl, &cc, NULL, 0)) return NULL;
    struct oref_mg *mg = (struct oref_mg *)calloc(1, sizeof *mg);
    mg->p = p;
    mg->mask = mask;
    mg->cache = cache;
    mg->work = work;
    mg->meanfree = meanfree;
    mg->nlevels = nl;
    mg->coarse_cells = cc;
    mg->levels = (level_t *)calloc(nl, sizeof(level_t));
    mg->coeff = (float *)calloc(LANES * (cc ? cc : 1), sizeof(float));
    mg->value = (float *)calloc(LANES * (cc ? cc : 1), sizeof(float));
    mg->temp = (float *)calloc(p->dims[3], sizeof(float));
    level_t *L0 = &mg->levels[0];
    memcpy(L0->dims, p->dims, sizeof L0->dims);
    memcpy(L0->child, p->dims, sizeof L0->child);
    memcpy(L0->faces, p->faces, sizeof L0->faces);
    L0->location[3] = p->flags[0];
    uint32_t offset = 0;
    for (uint32_t l = 1; l < nl; l++) {
        level_t *C = &mg->levels[l - 1], *L = &mg->levels[l];
        for (int a = 0; a < 3; a++) L->dims[a] = (C->dims[a] + 1) / 2;
        L->dims[3] = L->dims[0] * L->dims[1] * L->dims[2];
        memcpy(L->child, C->dims, sizeof L->child);
        memcpy(L->faces, p->faces, sizeof L->faces);
        L->location[0] = offset;
        L->location[1] = C->location[0];
        L->location[2] = l;
        L->location[3] = p->flags[0];
        offset += L->dims[3];
    }
    mg->groups = (p->dims[3] + 255u) / 256u;
    return mg;
}
static void mg_free(struct oref_mg *mg) {
    if (!mg) return;
    free(mg->levels);
    free(mg->coeff);
    free(mg->value);
    free(mg->temp);
    free(mg);
}
static void mg_build_all(struct oref_mg *mg) {
    for (uint32_t l = 1; l < mg->nlevels; l++) mg_build_level(mg, &mg->levels[l]);
}

/* ------------------------------------------------------------- anchors */
/* anchors(): src/fluid/mod.rs:1447-1493 */
uint32_t oref_anchors(uint32_t *mask, const uint32_t dims[3], uint32_t periodic_bits) {
    uint64_t n = (uint64_t)dims[0] * dims[1] * dims[2];
    uint32_t components = 0;
    uint32_t *roots = (uint32_t *)calloc(n ? n : 1, sizeof(uint32_t));
    uint32_t *queue = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    for (uint64_t root = 0; root < n; root++) {
        if (mask[root] != 1u) continue;
        components++;
        mask[root] = 4u;
        roots[root] = (uint32_t)root;
        uint64_t head = 0, tail = 0;
        queue[tail++] = (uint32_t)root;
        while (head < tail) {
            uint32_t i = queue[head++];
            uint32_t p[3] = {i % dims[0], (i / dims[0]) % dims[1], i / (dims[0] * dims[1])};
            for (int axis = 0; axis < 3; axis++)
                for (int dir = -1; dir <= 1; dir += 2) {
                    uint32_t q[3] = {p[0], p[1], p[2]};
                    int64_t v = (int64_t)p[axis] + dir;
                    if (periodic_bits & (1u << axis)) {
                        int64_t m = (int64_t)dims[axis];
                        v = ((v % m) + m) % m; /* rem_euclid */
                    } else if (v < 0 || v >= (int64_t)dims[axis]) {
                        continue;
                    }
                    q[axis] = (uint32_t)v;
                    uint64_t j = q[0] + (uint64_t)dims[0] * (q[1] + (uint64_t)dims[1] * q[2]);
                    if (mask[j] == 1u) {
                        mask[j] = 3u;
                        roots[j] = (uint32_t)root;
                        queue[tail++] = (uint32_t)j;
                    }
                }
        }
    }
    for (uint64_t i = 0; i < n; i++) {
        if (mask[i] == 3u) mask[i] = 1u | (roots[i] << 2);
        else if (mask[i] == 4u) mask[i] = 2u | (roots[i] << 2);
    }
    free(roots);
    free(queue);
    return components;
}

/* ------------------------------------------------------------- params */
void oref_make_params(oref_params *p, const uint32_t dims[3], float h, float dt, float rho_liquid,
                      float rho_air, int two_phase, uint32_t periodic_bits, float rel_tol,
                      float abs_div_tol, uint32_t fluid_cells, int thermal_drag, float drag_rate) {
    memset(p, 0, sizeof *p);
    for (int a = 0; a < 3; a++) {
        p->dims[a] = dims[a];
        p->faces[a] = dims[a] + 1;
    }
    p->dims[3] = dims[0] * dims[1] * dims[2];
    p->faces[3] = p->faces[0] * p->faces[1] * p->faces[2];
    p->flags[0] = periodic_bits;
    p->flags[3] = thermal_drag ? 1u : 0u;
    p->physical[0] = h;
    p->physical[1] = dt;
    p->physical[3] = rho_liquid;
    p->surface[0] = two_phase ? 1.0f : 0.0f;
    p->surface[1] = two_phase ? rho_air : rho_liquid;
    p->solve[0] = rel_tol * rel_tol;
    float h2 = h * h;
    p->solve[1] = (abs_div_tol * abs_div_tol) * (h2 * h2) * (float)fluid_cells;
    p->solve[2] = (float)fluid_cells;
    p->solve[3] = drag_rate;
}

/* ---------------------------------------------------------- project() */
static int read_convergence(const state *s, float *residual, int *converged, uint32_t *iterations) {
    const float *f = &s->scalars[0][0];
    float r = sqrtf(f[1] / fmaxf(f[2], 1e-38f));
    int bad = !isfinite(r) || f[1] < 0.0f || f[2] < 0.0f;
    for (int k = 0; k < 8; k++)
        if (!isfinite(f[k])) bad = 1;
    if (bad) return 2; /* "Nonfinite fluid pressure residual" */
    *residual = r;
    *converged = f[6] > 0.5f;
    *iterations = (uint32_t)f[7];
    return 0;
}
static void refresh_stages(state *s) {
    k_pressure_refresh(s);
    if (s->p->initial[3] > 0.0f) {
        k_pressure_residual_mean(s);
        k_project_pressure_residual(s, 1);
    }
    k_initial_reduce(s);
}
static void mg_initialize(struct oref_mg *mg, state *s) {
    mg_cycle(mg);
    mg_dot_partial(mg, 1);
    k_initial_reduce(s);
}
static void mg_iterate(struct oref_mg *mg, state *s, uint32_t batch) {
    for (uint32_t b = 0; b < batch; b++) {
        k_pressure_apply(s);
        k_alpha_reduce(s);
        k_update(s);
        if (s->p->initial[3] > 0.0f) {
            k_pressure_residual_mean(s);
            k_project_pressure_residual(s, 0);
        }
        mg_cycle(mg);
        mg_dot_partial(mg, 0);
        k_beta_reduce(s);
        mg_preconditioned_search(mg);
    }
}
static void jacobi_iterate(state *s, uint32_t batch, int meanfree) {
    for (uint32_t b = 0; b < batch; b++) {
        k_pressure_apply(s);
        k_alpha_reduce(s);
        k_update(s);
        if (meanfree) {
            k_pressure_residual_mean(s);
            k_project_pressure_residual(s, 0);
        }
        k_beta_reduce(s);
        k_search(s);
    }
}

void oref_project(const oref_params *params, const uint32_t *mask, uint32_t components, const float *occupancy,
                  const float *phase, const float *old_pressure, float *predicted, float *velocity, float *work,
                  uint32_t max_iterations, int warm_start, int force_mg, int force_meanfree, oref_result *res) {
    oref_params p = *params;
    uint32_t fluid_cells = 0;
    for (uint32_t i = 0; i < p.dims[3]; i++) fluid_cells += mask[i] != 0u;
    /* configure_pressure_projection: mod.rs:978-1002 */
    int meanfree = components == 1u;
    if (force_meanfree >= 0) meanfree = force_meanfree && components == 1u;
    uint32_t nf = fluid_cells ? fluid_cells : 1u;
    p.initial[3] = meanfree ? 1.0f / (float)nf : 0.0f;
    p.solve[2] = meanfree ? 1.0f : (float)nf;

    state s;
    memset(&s, 0, sizeof s);
    s.p = &p;
    s.mask = mask;
    s.occ = occupancy;
    s.phase = phase;
    s.oldp = old_pressure;
    s.velocity = velocity;
    s.predicted = predicted;
    s.work = work;
    s.groups = (p.dims[3] + 255u) / 256u;
    s.partials = (float *)calloc((size_t)LANES * s.groups, sizeof(float));
    memset(res, 0, sizeof *res);
    res->meanfree = meanfree;

    if (warm_start) k_pressure_warm(&s);
    k_pressure_coefficients(&s);
    k_pressure_guess(&s);
    refresh_stages(&s);
    uint32_t iterations = 0, it_read = 0;
    float residual = 0.0f;
    int conv = 0;
    int st = read_convergence(&s, &residual, &conv, &it_read);
    struct oref_mg *mg = NULL;
    int preferred = p.dims[3] >= 96u * 96u * 96u;
    if (force_mg >= 0) preferred = force_mg;
    if (st == 0 && preferred && !conv) {
        mg = mg_new(&p, mask, velocity, work, meanfree);
        if (mg) {
            mg->fluid_state = &s;
            mg->partials = s.partials;
            res->levels = mg->nlevels;
            res->coarse_cells = mg->coarse_cells;
        }
    }
    res->multigrid = mg != NULL;
    if (st == 0 && !conv && mg) {
        mg_build_all(mg);
        mg_initialize(mg, &s);
    }
    while (st == 0 && !conv && iterations < max_iterations) {
        uint32_t batch = mg ? 8u : 32u;
        if (batch > max_iterations - iterations) batch = max_iterations - iterations;
        if (batch > 64u - iterations % 64u) batch = 64u - iterations % 64u;
        if (mg) mg_iterate(mg, &s, batch);
        else jacobi_iterate(&s, batch, meanfree);
        st = read_convergence(&s, &residual, &conv, &it_read);
        if (st) break;
        if (it_read <= iterations && !conv) {
            st = 3; /* "Fluid pressure iteration made no progress" */
            break;
        }
        iterations = it_read;
        if (conv) {
            refresh_stages(&s);
            st = read_convergence(&s, &residual, &conv, &it_read);
            if (st) break;
            if (!conv && mg) mg_initialize(mg, &s);
        } else if (iterations % 64u == 0u || iterations == max_iterations) {
            k_pressure_check(&s);
            k_check_reduce(&s);
            st = read_convergence(&s, &residual, &conv, &it_read);
        }
    }
    if (st == 0 && !conv) st = 1; /* "did not converge after N iterations" */
    if (st == 0) {
        k_correct(&s);
        if (warm_start) k_pressure_commit(&s);
    }
    res->status = st;
    res->iterations = iterations;
    res->residual = residual;
    mg_free(mg);
    free(s.partials);
}

/* ----------------------------------------------------- standalone probes */
static state probe_state(const oref_params *p, const uint32_t *mask, const float *occ, const float *phase,
                         float *velocity, float *work) {
    state s;
    memset(&s, 0, sizeof s);
    s.p = p;
    s.mask = mask;
    s.occ = occ;
    s.phase = phase;
    s.velocity = velocity;
    s.work = work;
    s.groups = (p->dims[3] + 255u) / 256u;
    return s;
}
void oref_coefficients(const oref_params *params, const uint32_t *mask, const float *occupancy, const float *phase,
                       float *velocity) {
    state s = probe_state(params, mask, occupancy, phase, velocity, NULL);
    k_pressure_coefficients(&s);
}
void oref_apply_cached(const oref_params *params, const uint32_t *mask, const float *velocity, const float *work,
                       uint32_t kind, float *out) {
    state s = probe_state(params, mask, NULL, NULL, (float *)velocity, (float *)work);
    for (uint32_t i = 0; i < params->dims[3]; i++)
        out[i] = mask[i] ? apply_cached(&s, decode3(i, params->dims), kind) : 0.0f;
}
void oref_apply_uncached(const oref_params *params, const uint32_t *mask, const float *occupancy, const float *phase,
                         const float *work, uint32_t kind, float *out, float *diag_out) {
    state s = probe_state(params, mask, occupancy, phase, NULL, (float *)work);
    for (uint32_t i = 0; i < params->dims[3]; i++) {
        out[i] = diag_out[i] = 0.0f;
        if (!mask[i]) continue;
        ivec3 pos = decode3(i, params->dims);
        /* The reference's uncached probe (src/fluid/tests.rs:562-569):
           laplacian, with pinned anchors answering with their potential. */
        out[i] = pinned_anchor(&s, i) ? potential(&s, pos, kind) : laplacian(&s, pos, kind);
        diag_out[i] = diagonal(&s, pos);
    }
}
oref_mg *oref_mg_create(const oref_params *params, const uint32_t *mask, const float *velocity, int meanfree) {
    return mg_new(params, mask, velocity, NULL, meanfree);
}
void oref_mg_destroy(oref_mg *mg) { mg_free(mg); }
uint32_t oref_mg_levels(const oref_mg *mg, uint32_t *level_dims, uint32_t *offsets) {
    for (uint32_t l = 0; l < mg->nlevels; l++) {
        if (level_dims) memcpy(level_dims + 4 * l, mg->levels[l].dims, 4 * sizeof(uint32_t));
        if (offsets) offsets[l] = mg->levels[l].location[0];
    }
    return mg->nlevels;
}
void oref_mg_build(oref_mg *mg) { mg_build_all(mg); }
void oref_mg_apply(oref_mg *mg, float *work) {
    mg->work = work;
    mg_cycle(mg);
}
float *oref_mg_coeff(oref_mg *mg) { return mg->coeff; }
float *oref_mg_value(oref_mg *mg) { return mg->value; }
void oref_mg_probe_action(oref_mg *mg, uint32_t level, const float *work, float *predicted_w) {
    /* probe_action (multigrid_probes.wgsl:7) */
    mg->work = (float *)work;
    const level_t *L = &mg->levels[level];
    const int fine = L->location[2] == 0u;
    for (uint32_t i = 0; i < L->dims[3]; i++) {
        float a = mg_action(mg, L, decode3(i, L->dims), L->dims, L->location[0], fine, 0);
        if (fine) predicted_w[i] = a;
        else mg->value[LANES * (L->location[0] + i) + 2] = a;
    }
}
void oref_mg_coarse_solve(oref_mg *mg, float *work) {
    mg->work = work;
    mg_coarse_solve_level(mg, &mg->levels[mg->nlevels - 1]);
}
void oref_mg_coarse_jacobi_sequence(oref_mg *mg, float *work) {
    /* clear + COARSE_SWEEPS/2 x (smooth_to_temp, smooth_from_temp):
       multigrid/tests.rs:564-568 with multigrid_probes.wgsl:3-5 */
    mg->work = work;
    const level_t *L = &mg->levels[mg->nlevels - 1];
    for (uint32_t i = 0; i < L->dims[3]; i++) {
        if (L->location[2] == 0u) work[LANES * i + 3] = 0.0f;
        else mg->value[LANES * (L->location[0] + i) + 1] = 0.0f;
    }
    for (uint32_t k = 0; k < COARSE_SWEEPS / 2; k++) {
        mg_jacobi(mg, L, 0);
        mg_jacobi(mg, L, 1);
    }
}

/* ------------------------------------------- fluid step and fields
 * predict, viscous, fields and diagnostics of src/fluid/solver.wgsl
 * (:108-163, :256-291) for a step without a moving interface
 * (FluidState::step, src/fluid/mod.rs:1246-1333).  em: vec4 per cell, the
 * force density in .xyz (the force lanes of the EM result), or NULL;
 * acceleration: the body acceleration of Params.acceleration. */

/* em_force(): :108 */
static void em_force(const state *s, const float *em, ivec3 pos, float out[3]) {
    ivec3 q = wrap_cell(s, pos);
    out[0] = out[1] = out[2] = 0.0f;
    if (!em || !valid_cell(s, q)) return;
    const float *f = em + LANES * idx3(q, s->p->dims);
    out[0] = f[0];
    out[1] = f[1];
    out[2] = f[2];
}
/* sample_component()/sample_velocity(): :109-117, face(.., false) */
static float sample_component(const state *s, const float position[3], uint32_t axis) {
    float q[3];
    int32_t base[3];
    float fraction[3];
    for (int a = 0; a < 3; a++) {
        const float offset = (uint32_t)a == axis ? 0.0f : 0.5f;
        q[a] = position[a] - offset;
        const float fl = floorf(q[a]);
        base[a] = (int32_t)fl;
        fraction[a] = q[a] - fl; /* fract() */
    }
    float value = 0.0f;
    for (int z = 0; z < 2; z++)
        for (int y = 0; y < 2; y++)
            for (int x = 0; x < 2; x++) {
                const int o[3] = {x, y, z};
                float w[3];
                for (int a = 0; a < 3; a++) w[a] = o[a] > 0 ? fraction[a] : 1.0f - fraction[a];
                ivec3 c = {{base[0] + x, base[1] + y, base[2] + z}};
                value += face_value(s, c, axis, 0) * w[0] * w[1] * w[2];
            }
    return value;
}
static void sample_velocity(const state *s, const float position[3], float out[3]) {
    for (uint32_t a = 0; a < 3; a++) out[a] = sample_component(s, position, a);
}

/* predict(): :127-141.  flags.y: semi-Lagrangian RK2 advection. */
void oref_predict(const oref_params *params, const uint32_t *mask, const float *velocity, float *predicted) {
    state s;
    memset(&s, 0, sizeof s);
    s.p = params;
    s.mask = mask;
    s.velocity = (float *)velocity;
    const oref_params *p = params;
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)p->faces[3]; ii++) {
        const uint32_t i = (uint32_t)ii;
        const ivec3 pos = decode3(i, p->faces);
        float out[4] = {0, 0, 0, 0};
        for (uint32_t axis = 0; axis < 3; axis++) {
            if (!open_face(&s, pos, axis)) continue;
            const float center = face_value(&s, pos, axis, 0);
            float advected = center;
            if (p->flags[1] != 0u) {
                float at[3], v[3], mid[3], back[3], vm[3];
                for (int a = 0; a < 3; a++) at[a] = (float)pos.v[a] + 0.5f;
                at[axis] -= 0.5f;
                sample_velocity(&s, at, v);
                const float half = 0.5f * p->physical[1] / p->physical[0];
                for (int a = 0; a < 3; a++) mid[a] = at[a] - v[a] * half;
                sample_velocity(&s, mid, vm);
                const float full = p->physical[1] / p->physical[0];
                for (int a = 0; a < 3; a++) back[a] = at[a] - vm[a] * full;
                advected = sample_component(&s, back, axis);
            }
            out[axis] = advected;
        }
        memcpy(predicted + LANES * i, out, sizeof out);
    }
}

/* viscous(): :143-163 without a moving interface (surface.x = 0): explicit
 * Laplacian with mirrored (no-slip) closed tangential neighbours, body and EM
 * acceleration, times the face mobility. */
/* capillary_force(): :52-57, curvature per cell (reserved.w) or NULL */
static float capillary_force(const state *s, const float *curv, float sigma, ivec3 pos, uint32_t axis) {
    if (s->p->surface[0] < 0.5f || !open_face(s, pos, axis)) return 0.0f;
    ivec3 left = pos;
    left.v[axis] -= 1;
    const float al = occupancy(s, left), ar = occupancy(s, pos);
    const float kl = curv ? curv[idx3(wrap_cell(s, left), s->p->dims)] : 0.0f;
    const float kr = curv ? curv[idx3(wrap_cell(s, pos), s->p->dims)] : 0.0f;
    const float wl = al * (1.0f - al), wr = ar * (1.0f - ar);
    const float k = wl + wr > 1e-6f ? (wl * kl + wr * kr) / fmaxf(wl + wr, 1e-20f) : 0.5f * (kl + kr);
    return sigma * k * (ar - al) / s->p->physical[0];
}
void oref_viscous(const oref_params *params, const uint32_t *mask, const float *occupancy, const float *phase,
                  const float *em, const float acceleration[3], const float *predicted, float *velocity) {
    oref_viscous_surface(params, mask, occupancy, phase, em, acceleration, NULL, 0.0f, predicted, velocity);
}
void oref_viscous_surface(const oref_params *params, const uint32_t *mask, const float *occupancy, const float *phase,
                          const float *em, const float acceleration[3], const float *curvature, float sigma,
                          const float *predicted, float *velocity) {
    state s;
    memset(&s, 0, sizeof s);
    s.p = params;
    s.mask = mask;
    s.occ = occupancy;
    s.phase = phase;
    s.predicted = (float *)predicted;
    const oref_params *p = params;
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)p->faces[3]; ii++) {
        const uint32_t i = (uint32_t)ii;
        const ivec3 pos = decode3(i, p->faces);
        float out[4] = {0, 0, 0, 0};
        for (uint32_t axis = 0; axis < 3; axis++) {
            if (!open_face(&s, pos, axis)) continue;
            const float center = face_value(&s, pos, axis, 1);
            float laplace = 0.0f;
            if (p->surface[0] < 0.5f)
                for (uint32_t d = 0; d < 3; d++)
                    for (int sign = -1; sign <= 1; sign += 2) {
                        ivec3 q = pos;
                        q.v[d] += sign;
                        float neighbor = face_value(&s, q, axis, 1);
                        if (!open_face(&s, q, axis) && d != axis) neighbor = -center;
                        laplace += neighbor - center;
                    }
            ivec3 left = pos;
            left.v[axis] -= 1;
            float rho = p->physical[3], capillary = 0.0f;
            if (p->surface[0] > 0.5f) {
                rho = face_density(&s, pos, axis);
                capillary = capillary_force(&s, curvature, sigma, pos, axis) / rho;
            }
            float el[3], er[3];
            em_force(&s, em, left, el);
            em_force(&s, em, pos, er);
            const float acc = acceleration[axis] + (el[axis] + er[axis]) / (2.0f * rho) + capillary;
            float beta = mobility(&s, pos, axis);
            if (p->surface[0] > 0.5f) beta *= rho / p->physical[3];
            out[axis] = (center + p->physical[2] * p->physical[1] / (p->physical[0] * p->physical[0]) * laplace +
                         p->physical[1] * acc) *
                        beta;
        }
        memcpy(velocity + LANES * i, out, sizeof out);
    }
}

/* fields() and diagnostics(): :256-291.  cells: 16 floats per cell (velocity
 * xyz + speed, pressure + divergence, force, reserved) or NULL.  reserved_in:
 * vec4 per cell, the cells' previous reserved lanes (y phase fraction, z
 * liquid fraction, w curvature), or NULL for zeros.  scalars: the 12 floats
 * diagnostics writes to scalars[2..4]. */
void oref_fields(const oref_params *params, const uint32_t *mask, const float *occupancy, const float *work,
                 const float *velocity, const float *em, const float acceleration[3], const float *reserved_in,
                 float *cells, float scalars[12]) {
    state s;
    memset(&s, 0, sizeof s);
    s.p = params;
    s.mask = mask;
    s.occ = occupancy;
    s.velocity = (float *)velocity;
    s.work = (float *)work;
    const oref_params *p = params;
    const uint32_t groups = (p->dims[3] + 255u) / 256u;
    float *part = (float *)calloc((size_t)3 * LANES * (groups ? groups : 1), sizeof(float));
#pragma omp parallel for schedule(static)
    for (int64_t gg = 0; gg < (int64_t)groups; gg++) {
        float ra[256][4], rb[256][4], rc[256][4];
        for (uint32_t l = 0; l < 256u; l++) {
            const uint32_t i = (uint32_t)gg * 256u + l;
            float stats[4] = {0, 0, 0, 0}, other[4] = {0, 0, 0, 0};
            float max_face = 0.0f, melt = 0.0f;
            if (i < p->dims[3]) {
                float out[16];
                memset(out, 0, sizeof out);
                const float *old = reserved_in ? reserved_in + LANES * i : NULL;
                const float oy = old ? old[1] : 0.0f, oz = old ? old[2] : 0.0f, ow = old ? old[3] : 0.0f;
                if (p->surface[0] > 0.5f) {
                    out[13] = oy;
                    out[14] = oz;
                    out[15] = ow;
                }
                if (mask[i] != 0u) {
                    const ivec3 pos = decode3(i, p->dims);
                    float v[3] = {0, 0, 0}, face_energy = 0.0f;
                    for (uint32_t axis = 0; axis < 3; axis++) {
                        ivec3 q = pos;
                        q.v[axis] += 1;
                        const float a = face_value(&s, pos, axis, 0), b = face_value(&s, q, axis, 0);
                        v[axis] = 0.5f * (a + b);
                        face_energy += 0.5f * (a * a + b * b);
                        max_face = fmaxf(max_face, fmaxf(fabsf(face_value(&s, pos, axis, 0)),
                                                         fabsf(face_value(&s, q, axis, 0))));
                    }
                    melt = p->flags[3] != 0u ? oy : 1.0f;
                    if (p->surface[0] > 0.5f) melt *= oz;
                    const float speed = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                    const float div = divergence(&s, pos, 0);
                    const float x = work[LANES * i];
                    const float potential_value =
                        mean_free_pressure(&s) ? x - work[LANES * (mask[i] >> 2u)] : x;
                    const float pressure = potential_value * p->physical[3] / p->physical[1];
                    float force[3];
                    em_force(&s, em, pos, force);
                    for (int a = 0; a < 3; a++) force[a] = p->physical[3] * acceleration[a] + force[a];
                    out[0] = v[0];
                    out[1] = v[1];
                    out[2] = v[2];
                    out[3] = speed;
                    out[4] = pressure;
                    out[5] = div;
                    out[8] = force[0];
                    out[9] = force[1];
                    out[10] = force[2];
                    out[12] = 1.0f;
                    out[13] = p->flags[3] != 0u ? oy : 1.0f;
                    out[14] = oz;
                    out[15] = ow;
                    int bad = v[0] != v[0] || v[1] != v[1] || v[2] != v[2];
                    bad = bad || force[0] != force[0] || force[1] != force[1] || force[2] != force[2];
                    bad = bad || fabsf(force[0]) > 1e30f || fabsf(force[1]) > 1e30f || fabsf(force[2]) > 1e30f;
                    bad = bad || speed > 1e25f || !(fabsf(pressure) < 1e30f) || !(fabsf(div) < 1e30f);
                    const float rho = p->surface[0] > 0.5f ? density(&s, pos) : p->physical[3];
                    stats[0] = speed;
                    stats[1] = fabsf(div);
                    stats[2] = div * div;
                    stats[3] = 0.5f * rho * face_energy * p->physical[0] * p->physical[0] * p->physical[0];
                    other[0] = fabsf(pressure);
                    other[1] = div;
                    other[2] = sqrtf(force[0] * force[0] + force[1] * force[1] + force[2] * force[2]);
                    other[3] = bad ? 1.0f : 0.0f;
                }
                if (cells) memcpy(cells + 16 * (size_t)i, out, sizeof out);
            }
            memcpy(ra[l], stats, sizeof stats);
            memcpy(rb[l], other, sizeof other);
            rc[l][0] = max_face;
            rc[l][1] = melt;
            rc[l][2] = rc[l][3] = 0.0f;
        }
        for (uint32_t st = 128u; st > 0u; st /= 2u)
            for (uint32_t l = 0; l < st; l++) {
                ra[l][0] = fmaxf(ra[l][0], ra[l + st][0]);
                ra[l][1] = fmaxf(ra[l][1], ra[l + st][1]);
                ra[l][2] += ra[l + st][2];
                ra[l][3] += ra[l + st][3];
                rb[l][0] = fmaxf(rb[l][0], rb[l + st][0]);
                rb[l][1] += rb[l + st][1];
                rb[l][2] = fmaxf(rb[l][2], rb[l + st][2]);
                rb[l][3] += rb[l + st][3];
                rc[l][0] = fmaxf(rc[l][0], rc[l + st][0]);
                rc[l][1] += rc[l + st][1];
                rc[l][2] = rc[l][3] = 0.0f;
            }
        memcpy(part + LANES * gg, ra[0], 4 * sizeof(float));
        memcpy(part + LANES * (groups + gg), rb[0], 4 * sizeof(float));
        memcpy(part + LANES * (2 * groups + gg), rc[0], 4 * sizeof(float));
    }
    /* diagnostics(): one workgroup, 256-stride loop, then the tree */
    float ra[256][4], rb[256][4], rc[256][4];
    for (uint32_t l = 0; l < 256u; l++) {
        float a[4] = {0, 0, 0, 0}, b[4] = {0, 0, 0, 0}, c[4] = {0, 0, 0, 0};
        for (uint32_t i = l; i < groups; i += 256u) {
            const float *fs = part + LANES * (2 * groups + i), *x = part + LANES * i, *y = part + LANES * (groups + i);
            c[0] = fmaxf(c[0], fs[0]);
            c[1] = c[1] + fs[1];
            a[0] = fmaxf(a[0], x[0]);
            a[1] = fmaxf(a[1], x[1]);
            a[2] = a[2] + x[2];
            a[3] = a[3] + x[3];
            b[0] = fmaxf(b[0], y[0]);
            b[1] = b[1] + y[1];
            b[2] = fmaxf(b[2], y[2]);
            b[3] = b[3] + y[3];
        }
        memcpy(ra[l], a, sizeof a);
        memcpy(rb[l], b, sizeof b);
        memcpy(rc[l], c, sizeof c);
    }
    for (uint32_t st = 128u; st > 0u; st /= 2u)
        for (uint32_t l = 0; l < st; l++) {
            ra[l][0] = fmaxf(ra[l][0], ra[l + st][0]);
            ra[l][1] = fmaxf(ra[l][1], ra[l + st][1]);
            ra[l][2] += ra[l + st][2];
            ra[l][3] += ra[l + st][3];
            rb[l][0] = fmaxf(rb[l][0], rb[l + st][0]);
            rb[l][1] += rb[l + st][1];
            rb[l][2] = fmaxf(rb[l][2], rb[l + st][2]);
            rb[l][3] += rb[l + st][3];
            rc[l][0] = fmaxf(rc[l][0], rc[l + st][0]);
            rc[l][1] += rc[l + st][1];
            rc[l][2] = rc[l][3] = 0.0f;
        }
    memcpy(scalars, ra[0], 4 * sizeof(float));
    memcpy(scalars + 4, rb[0], 4 * sizeof(float));
    memcpy(scalars + 8, rc[0], 4 * sizeof(float));
    free(part);
}

/* ----------------------------------------- moving-interface stresses
 * src/fluid/viscosity.wgsl and stabilized.wgsl with the host sequencing of
 * FluidState::diffuse_surface_stress (src/fluid/mod.rs:1160-1240) and
 * stabilized::schedule/encode (src/fluid/stabilized.rs).  The per-cell lanes
 * the shaders borrow from the display packet (pressure.w viscosity,
 * pressure.y/z shear, velocity/force RKC initial state) are separate arrays
 * here. */
typedef struct {
    state s;
    float mu_air;
    float *mu;    /* cached cell viscosity */
    float *t4;    /* xx, yy, zz, xy per cell */
    float *t2;    /* xz, yz per cell */
    float *y0;    /* 4 per cell */
    float *f0;    /* 4 per cell */
} stress_state;

static ivec3 shifted(ivec3 q, uint32_t a, int d) {
    q.v[a] += d;
    return q;
}
static float dynamic_mu(const stress_state *S, ivec3 q) {
    if (!fluid(&S->s, q)) return 0.0f;
    const float t = fminf(fmaxf(occupancy(&S->s, q), 0.0f), 1.0f);
    const float mu_l = S->s.p->physical[2] * S->s.p->physical[3];
    return S->mu_air * (1.0f - t) + mu_l * t;
}
static float coefficient_mu(const stress_state *S, ivec3 q, int cached) {
    if (!cached) return dynamic_mu(S, q);
    ivec3 at = wrap_cell(&S->s, q);
    if (!valid_cell(&S->s, at)) return 0.0f;
    return S->mu[idx3(at, S->s.p->dims)];
}
static float edge_mu_c(const stress_state *S, ivec3 q, uint32_t i, uint32_t j, int cached) {
    float total = 0.0f, count = 0.0f;
    for (int a = 0; a < 2; a++)
        for (int b = 0; b < 2; b++) {
            ivec3 at = q;
            at.v[i] -= a;
            at.v[j] -= b;
            if (fluid(&S->s, at)) {
                total += coefficient_mu(S, at, cached);
                count += 1.0f;
            }
        }
    return total / fmaxf(count, 1.0f);
}
static float sface(const stress_state *S, ivec3 q, uint32_t i) { return face_value(&S->s, q, i, 1); }
static float normal_stress(const stress_state *S, ivec3 q, uint32_t i, int cached) {
    if (!fluid(&S->s, q)) return 0.0f;
    return 2.0f * coefficient_mu(S, q, cached) * (sface(S, shifted(q, i, 1), i) - sface(S, q, i)) /
           S->s.p->physical[0];
}
static float shear_stress(const stress_state *S, ivec3 q, uint32_t i, uint32_t j, int cached) {
    const ivec3 lower_i = shifted(q, j, -1), lower_j = shifted(q, i, -1);
    float ui1 = sface(S, q, i), ui0 = sface(S, lower_i, i);
    float uj1 = sface(S, q, j), uj0 = sface(S, lower_j, j);
    if (!open_face(&S->s, q, i) && open_face(&S->s, lower_i, i)) ui1 = -ui0;
    if (!open_face(&S->s, lower_i, i) && open_face(&S->s, q, i)) ui0 = -ui1;
    if (!open_face(&S->s, q, j) && open_face(&S->s, lower_j, j)) uj1 = -uj0;
    if (!open_face(&S->s, lower_j, j) && open_face(&S->s, q, j)) uj0 = -uj1;
    return edge_mu_c(S, q, i, j, cached) * (ui1 - ui0 + uj1 - uj0) / S->s.p->physical[0];
}
static float tensor_normal(const stress_state *S, ivec3 q, uint32_t i) {
    ivec3 at = wrap_cell(&S->s, q);
    if (!valid_cell(&S->s, at)) return 0.0f;
    return S->t4[4 * (size_t)idx3(at, S->s.p->dims) + i];
}
static float tensor_shear(const stress_state *S, ivec3 q, uint32_t i, uint32_t j) {
    ivec3 at = wrap_cell(&S->s, q);
    if (!valid_cell(&S->s, at)) return shear_stress(S, q, i, j, 1);
    const size_t c = idx3(at, S->s.p->dims);
    const uint32_t plane = i + j;
    if (plane == 1u) return S->t4[4 * c + 3];
    return S->t2[2 * c + (plane - 2u)];
}
static float stress_acceleration(const stress_state *S, ivec3 q, uint32_t i, int cached) {
    const ivec3 left = shifted(q, i, -1);
    float divergence = 0.0f;
    if (cached) {
        divergence = tensor_normal(S, q, i) - tensor_normal(S, left, i);
        for (uint32_t j = 0; j < 3; j++)
            if (j != i) divergence += tensor_shear(S, shifted(q, j, 1), i, j) - tensor_shear(S, q, i, j);
    } else {
        divergence = normal_stress(S, q, i, 0) - normal_stress(S, left, i, 0);
        for (uint32_t j = 0; j < 3; j++)
            if (j != i) divergence += shear_stress(S, shifted(q, j, 1), i, j, 0) - shear_stress(S, q, i, j, 0);
    }
    return divergence / (S->s.p->physical[0] * face_density(&S->s, q, i));
}
static void k_stress_coefficients(stress_state *S) {
    const oref_params *p = S->s.p;
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)p->dims[3]; ii++) S->mu[ii] = dynamic_mu(S, decode3((uint32_t)ii, p->dims));
}
static void k_stress_tensor(stress_state *S) {
    const oref_params *p = S->s.p;
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)p->dims[3]; ii++) {
        const ivec3 q = decode3((uint32_t)ii, p->dims);
        float *t = S->t4 + 4 * ii;
        t[0] = normal_stress(S, q, 0, 1);
        t[1] = normal_stress(S, q, 1, 1);
        t[2] = normal_stress(S, q, 2, 1);
        t[3] = shear_stress(S, q, 0, 1, 1);
        S->t2[2 * ii] = shear_stress(S, q, 0, 2, 1);
        S->t2[2 * ii + 1] = shear_stress(S, q, 1, 2, 1);
    }
}
static void k_stress_save_initial(stress_state *S) {
    const oref_params *p = S->s.p;
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)p->dims[3]; ii++) {
        const ivec3 q = decode3((uint32_t)ii, p->dims);
        float y[4] = {0, 0, 0, 0}, op[4] = {0, 0, 0, 0};
        for (uint32_t axis = 0; axis < 3; axis++)
            if (open_face(&S->s, q, axis)) {
                y[axis] = sface(S, q, axis);
                op[axis] = stress_acceleration(S, q, axis, 1);
            }
        memcpy(S->y0 + 4 * ii, y, sizeof y);
        memcpy(S->f0 + 4 * ii, op, sizeof op);
    }
}
/* stress_stabilized: out (the velocity binding) = blend of the previous stage
 * (predicted binding), the stage before (out's old content), the initial
 * state and the operators. */
static void k_stress_stabilized(stress_state *S, const float row[8], float *out) {
    const oref_params *p = S->s.p;
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)p->faces[3]; ii++) {
        const uint32_t i = (uint32_t)ii;
        const ivec3 q = decode3(i, p->faces);
        float older[4], res[4] = {0, 0, 0, 0};
        memcpy(older, out + LANES * i, sizeof older);
        for (uint32_t axis = 0; axis < 3; axis++)
            if (open_face(&S->s, q, axis)) {
                const size_t cell = idx3(wrap_cell(&S->s, q), p->dims);
                const float previous = sface(S, q, axis);
                const float initial = S->y0[4 * cell + axis], initial_op = S->f0[4 * cell + axis];
                res[axis] = row[0] * previous + row[1] * older[axis] + row[2] * initial +
                            row[3] * stress_acceleration(S, q, axis, 1) + row[4] * initial_op;
            }
        memcpy(out + LANES * i, res, sizeof res);
    }
}
static void k_stress_diffuse(stress_state *S, float dt_sub, float *out) {
    const oref_params *p = S->s.p;
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)p->faces[3]; ii++) {
        const uint32_t i = (uint32_t)ii;
        const ivec3 q = decode3(i, p->faces);
        float res[4] = {0, 0, 0, 0};
        for (uint32_t axis = 0; axis < 3; axis++)
            if (open_face(&S->s, q, axis)) res[axis] = sface(S, q, axis) + dt_sub * stress_acceleration(S, q, axis, 0);
        memcpy(out + LANES * i, res, sizeof res);
    }
}
static float k_viscosity_bound(stress_state *S) {
    const oref_params *p = S->s.p;
    float best = 0.0f;
#pragma omp parallel for schedule(static) reduction(max : best)
    for (int64_t ii = 0; ii < (int64_t)p->faces[3]; ii++) {
        const ivec3 q = decode3((uint32_t)ii, p->faces);
        for (uint32_t c = 0; c < 3; c++)
            if (open_face(&S->s, q, c)) {
                const ivec3 left = shifted(q, c, -1);
                float sum = dynamic_mu(S, q) + dynamic_mu(S, left);
                for (uint32_t j = 0; j < 3; j++)
                    if (j != c) sum += edge_mu_c(S, q, c, j, 0) + edge_mu_c(S, shifted(q, j, 1), c, j, 0);
                const float b = 4.0f * sum / (face_density(&S->s, q, c) * p->physical[0] * p->physical[0]);
                if (b > best) best = b;
            }
    }
    return best;
}

/* stabilized::schedule (src/fluid/stabilized.rs:11-50): damped RKC2 rows
 * (mu, nu, 1-mu-nu, operator time, initial-operator time) for `euler_steps`
 * equivalent Euler steps of dt.  Returns the row count (<= cap). */
#define RKC_DAMPING 0.05
static uint32_t rkc_capacity(uint32_t euler_limit) { return (uint32_t)ceil(3.0 * sqrt((double)euler_limit)) + 2u; }
uint32_t oref_rkc_schedule(double dt, uint32_t euler_steps, float *rows, uint32_t cap) {
    const double stiffness = 1.8 * (double)euler_steps;
    const uint32_t smax = rkc_capacity(euler_steps);
    double *t = (double *)malloc((smax + 2) * sizeof(double)), *d = (double *)malloc((smax + 2) * sizeof(double));
    double *dd = (double *)malloc((smax + 2) * sizeof(double)), *b = (double *)malloc((smax + 2) * sizeof(double));
    uint32_t out = 0;
    for (uint32_t stages = 2; stages <= smax; stages++) {
        const double w0 = 1.0 + RKC_DAMPING / ((double)stages * (double)stages);
        t[0] = 1.0; t[1] = w0; d[0] = 0.0; d[1] = 1.0; dd[0] = 0.0; dd[1] = 0.0;
        for (uint32_t j = 2; j <= stages; j++) {
            t[j] = 2.0 * w0 * t[j - 1] - t[j - 2];
            d[j] = 2.0 * t[j - 1] + 2.0 * w0 * d[j - 1] - d[j - 2];
            dd[j] = 4.0 * d[j - 1] + 2.0 * w0 * dd[j - 1] - dd[j - 2];
        }
        const double w1 = d[stages] / dd[stages];
        if (stiffness > 0.9 * (1.0 + w0) / w1) continue;
        for (uint32_t j = 0; j <= stages; j++) b[j] = 0.0;
        for (uint32_t j = 2; j <= stages; j++) b[j] = dd[j] / (d[j] * d[j]);
        b[0] = b[2];
        b[1] = b[2];
        if (cap < stages) break;
        float *r = rows;
        memset(r, 0, 8 * sizeof(float));
        r[0] = 1.0f;
        r[3] = (float)(dt * b[1] * w1);
        out = 1;
        for (uint32_t j = 2; j <= stages; j++) {
            const float mu = (float)(2.0 * w0 * b[j] / b[j - 1]);
            const float nu = (float)(-b[j] / b[j - 2]);
            const double op = dt * 2.0 * w1 * b[j] / b[j - 1];
            const double a = 1.0 - b[j - 1] * t[j - 1];
            r = rows + 8 * out;
            memset(r, 0, 8 * sizeof(float));
            r[0] = mu;
            r[1] = nu;
            r[2] = 1.0f - mu - nu;
            r[3] = (float)op;
            r[4] = (float)(-a * op);
            out++;
        }
        break;
    }
    free(t); free(d); free(dd); free(b);
    return out;
}

/* FluidState::diffuse_surface_stress on the face records: `predicted` holds
 * the stage input (the predicted velocity) and receives the diffused
 * velocity; `velocity` holds the step's starting velocity (the RKC stages
 * alternate the two buffers as the reference does).  Returns 0, 1 for a
 * non-finite bound, 2 for too many substeps; *substeps the Euler substeps or
 * RKC stages run. */
int oref_diffuse_surface_stress(const oref_params *params, const uint32_t *mask, const float *occupancy,
                                const float *phase, float mu_air, float dt, uint32_t max_substeps,
                                float *predicted, float *velocity, uint32_t *substeps, float *gpu_bound) {
    stress_state S;
    memset(&S, 0, sizeof S);
    S.s.p = params;
    S.s.mask = mask;
    S.s.occ = occupancy;
    S.s.phase = phase;
    S.mu_air = mu_air;
    const uint32_t n = params->dims[3], nf = params->faces[3];
    *substeps = 0;
    if (gpu_bound) *gpu_bound = -1.0f;
    /* global_viscous_bound (src/fluid/mod.rs:1146-1159) */
    const double liquid = params->physical[3], ambient = params->surface[1];
    const double slack = (double)1e-5f + 4.0 * (double)1.1920929e-7f;
    const double floor_rho = fmin(liquid, ambient) - fabs(liquid - ambient) * slack;
    const double mu = (double)fmaxf(params->physical[2] * params->physical[3], mu_air);
    const double h = params->physical[0];
    double count;
    if (floor_rho > 0.0 && (double)dt * (24.0 * mu / (floor_rho * h * h) * (1.0 + 32.0 * (double)1.1920929e-7f)) <= 1.8) {
        const double bound = 24.0 * mu / (floor_rho * h * h) * (1.0 + 32.0 * (double)1.1920929e-7f);
        if (bound == 0.0) return 0;
        count = 1.0;
    } else {
        const float bound = k_viscosity_bound(&S);
        if (gpu_bound) *gpu_bound = bound;
        if (!isfinite(bound) || bound < 0.0f) return 1;
        if (bound == 0.0f) return 0;
        count = fmax(ceil((double)dt * (double)bound / 1.8), 1.0);
    }
    if (count > (double)max_substeps) return 2;
    const uint32_t steps = (uint32_t)count;
    S.mu = (float *)calloc(n, sizeof(float));
    S.t4 = (float *)calloc((size_t)4 * n, sizeof(float));
    S.t2 = (float *)calloc((size_t)2 * n, sizeof(float));
    S.y0 = (float *)calloc((size_t)4 * n, sizeof(float));
    S.f0 = (float *)calloc((size_t)4 * n, sizeof(float));
    if (steps > 8u) {
        const uint32_t cap = rkc_capacity(steps);
        float *rows = (float *)calloc((size_t)8 * cap, sizeof(float));
        const uint32_t nrows = oref_rkc_schedule((double)dt, steps, rows, cap);
        float *bufs[2] = {velocity, predicted}; /* parity 0: velocity binding, predicted binding */
        S.s.velocity = bufs[0];
        S.s.predicted = bufs[1];
        k_stress_coefficients(&S);
        k_stress_tensor(&S);
        k_stress_save_initial(&S);
        for (uint32_t i = 0; i < nrows; i++) {
            const uint32_t par = i % 2u;
            S.s.velocity = par ? bufs[1] : bufs[0];
            S.s.predicted = par ? bufs[0] : bufs[1];
            if (i > 0) k_stress_tensor(&S);
            k_stress_stabilized(&S, rows + 8 * i, S.s.velocity);
        }
        if (nrows % 2u == 1u) memcpy(predicted, velocity, (size_t)LANES * nf * sizeof(float));
        *substeps = nrows;
        free(rows);
    } else {
        const float dt_sub = (float)((double)dt / (double)steps);
        S.s.predicted = predicted;
        for (uint32_t k = 0; k < steps; k++) {
            k_stress_diffuse(&S, dt_sub, velocity);
            memcpy(predicted, velocity, (size_t)LANES * nf * sizeof(float));
        }
        *substeps = steps;
    }
    free(S.mu); free(S.t4); free(S.t2); free(S.y0); free(S.f0);
    return 0;
}

/* ---- phase / surface classification (src/fluid/phase.wgsl:10-31) ----
 * The mobility mask and FluidCell.reserved lanes from the material ids, the
 * thermal phase (stride in floats; state.y of the reference's 16-float
 * packet) and the interface field (a, y at floats 0 and 1 of each record).
 * interface == NULL runs the `phase` pass, else the `surface` pass.
 * Returns the changed flags: bit 0 mobility changed, bit 1 a fraction
 * outside [-1e-5, 1+1e-5] or not finite (src/surface.rs:12). */
uint32_t oref_classify_cells(uint32_t n, const uint32_t *materials, uint32_t liquid, const float *thermal,
                             uint32_t thermal_stride, const float *interface, uint32_t interface_stride,
                             uint32_t *mask, float *cells) {
    uint32_t changed = 0;
    const float eps = 1e-5f;
    for (uint32_t i = 0; i < n; i++) {
        int mobile;
        if (!interface) {
            float fraction = 0.0f;
            if (materials[i] == liquid) fraction = thermal[(size_t)i * thermal_stride];
            mobile = fraction > 1e-6f;
            cells[(size_t)i * 16 + 13] = fraction;
        } else {
            float a = interface[(size_t)i * interface_stride];
            if (!(a >= -eps && a <= 1.0f + eps)) {
                changed |= 2u;
                continue;
            }
            float f = 1.0f;
            if (thermal && a > 0.0f) f = thermal[(size_t)i * thermal_stride];
            int wall = materials[i] != 0u && materials[i] != liquid;
            mobile = !wall && !(a > 0.0f && f <= 1e-6f);
            float *r = cells + (size_t)i * 16 + 12;
            r[0] = 1.0f;
            r[1] = f;
            r[2] = a;
            r[3] = interface[(size_t)i * interface_stride + 1];
        }
        int old = mask[i] != 0u;
        if (mobile != old) {
            mask[i] = mobile ? 1u : 0u;
            changed |= 1u;
        }
    }
    return changed;
}
