/*
 * oracle_native.c -- FP64 oracle for the GB300 projection's discrete problem.
 *
 * TEST INFRASTRUCTURE ONLY (see mhd_oracle.h).
 *
 * The discrete problem is the reference's variable-density MAC projection
 * (mobility beta = rho_l / mean face density, src/fluid/solver.wgsl:41-51;
 * b = -h^2 div u*, :104-107; u = u* - beta grad(phi)/h, :245-250) with three
 * differences that the GB300 path adds: face velocities are SoA arrays of
 * sizes (nx+1)ny nz, nx(ny+1)nz, nx ny(nz+1); the top z-face may be a
 * Dirichlet outlet (p = 0 on the face, i.e. conductance 2*beta to a zero
 * value half a cell away); components without an outlet are pinned at their
 * first cell (the root of src/fluid/mod.rs:1447-1493) by moving the edges to
 * that cell into the neighbours' diagonal ("reaction") terms.
 *
 * Mobilities are computed in FP32 with a fixed operation order (the GPU uses
 * the same order with rounding-explicit intrinsics), then the system is solved
 * in FP64 by conjugate gradients preconditioned with the same aggregation
 * V-cycle the GPU uses, taken in exact FP64 arithmetic, to ||b-Ax|| <= rtol ||b||.
 */
#include "mhd_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct { uint32_t d[3]; uint32_t periodic; } lvl_dims;

static inline int outlet_on(const onat_grid *g) { return g->outlet && !(g->periodic & 4u); }
static inline int64_t nbr(const uint32_t *d, uint32_t periodic, uint32_t x, uint32_t y, uint32_t z, int axis,
                          int dir) {
    int64_t c[3] = {x, y, z};
    c[axis] += dir;
    if (c[axis] < 0 || c[axis] >= (int64_t)d[axis]) {
        if (!(periodic & (1u << axis))) return -1;
        c[axis] = (c[axis] + d[axis]) % d[axis];
    }
    return c[0] + (int64_t)d[0] * (c[1] + (int64_t)d[1] * c[2]);
}

/* ------------------------------------------------------------ classes */
uint32_t onat_classify(const onat_grid *g, const uint8_t *solid, uint8_t *cls) {
    const uint32_t d[3] = {g->nx, g->ny, g->nz};
    const uint64_t n = (uint64_t)g->nx * g->ny * g->nz;
    uint32_t *queue = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    uint8_t *seen = (uint8_t *)calloc(n ? n : 1, 1);
    uint32_t pinned = 0;
    for (uint64_t i = 0; i < n; i++) cls[i] = solid[i] ? 0 : 1;
    for (uint64_t root = 0; root < n; root++) {
        if (cls[root] == 0 || seen[root]) continue;
        uint64_t head = 0, tail = 0;
        int touches = 0;
        seen[root] = 1;
        queue[tail++] = (uint32_t)root;
        while (head < tail) {
            uint32_t i = queue[head++];
            uint32_t x = i % d[0], y = (i / d[0]) % d[1], z = i / (d[0] * d[1]);
            if (outlet_on(g) && z == d[2] - 1) touches = 1;
            for (int a = 0; a < 3; a++)
                for (int dir = -1; dir <= 1; dir += 2) {
                    int64_t j = nbr(d, g->periodic, x, y, z, a, dir);
                    if (j < 0 || cls[j] == 0 || seen[j]) continue;
                    seen[j] = 1;
                    queue[tail++] = (uint32_t)j;
                }
        }
        if (!touches) {
            cls[root] = 2;
            pinned++;
        }
    }
    free(queue);
    free(seen);
    return pinned;
}

/* ------------------------------------------------------- coefficients */
static inline float nrho(const onat_grid *g, float a) { return g->rho_air * (1.0f - a) + g->rho_liquid * a; }
/* mobility() of src/fluid/solver.wgsl:43-51 for the face between cells L and
 * R: rho_l / mean face density (1 with one phase), divided by 1 + dt * drag
 * with drag = rate (1 - f)^2 / (f^3 + 1e-3), f the smaller thermal phase
 * fraction of the two cells, when a phase field is set.  FP32 in the
 * reference's operation order (built without contraction). */
static inline float nbeta(const onat_grid *g, const float *alpha, uint64_t L, uint64_t R) {
    float b = g->single ? 1.0f : g->rho_liquid / (0.5f * (nrho(g, alpha[L]) + nrho(g, alpha[R])));
    if (g->phase) {
        float f = fminf(g->phase[L], g->phase[R]);
        float drag = g->drag_rate * (1.0f - f) * (1.0f - f) / (f * f * f + 1e-3f);
        b = b / (1.0f + g->dt * drag);
    }
    return b;
}
void onat_coefficients(const onat_grid *g, const float *alpha, const uint8_t *cls, float *coef, float *gtop) {
    const uint32_t d[3] = {g->nx, g->ny, g->nz};
    const uint64_t n = (uint64_t)g->nx * g->ny * g->nz;
    for (uint64_t i = 0; i < (uint64_t)g->nx * g->ny; i++) gtop[i] = 0.0f;
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)n; ii++) {
        uint64_t i = (uint64_t)ii;
        uint32_t x = i % d[0], y = (i / d[0]) % d[1], z = (uint32_t)(i / ((uint64_t)d[0] * d[1]));
        float c[4] = {0, 0, 0, 0};
        if (cls[i] == 1) {
            for (int a = 0; a < 3; a++) {
                int64_t l = nbr(d, g->periodic, x, y, z, a, -1);
                if (l >= 0 && cls[l] == 1) c[a] = nbeta(g, alpha, (uint64_t)l, i);
            }
            float r = 0.0f;
            for (int a = 0; a < 3; a++)
                for (int dir = -1; dir <= 1; dir += 2) {
                    int64_t j = nbr(d, g->periodic, x, y, z, a, dir);
                    if (j >= 0 && cls[j] == 2) r += nbeta(g, alpha, i, (uint64_t)j);
                }
            if (outlet_on(g) && z == d[2] - 1) {
                float gt = 2.0f * nbeta(g, alpha, i, i);
                r += gt;
                gtop[x + (uint64_t)d[0] * y] = gt;
            }
            c[3] = r;
        }
        memcpy(coef + 4 * i, c, sizeof c);
    }
}

/* --------------------------------------------------------- operators */
static void rhs_d(const onat_grid *g, const uint8_t *cls, const double *u, const double *v, const double *w,
                  double *b) {
    const uint32_t nx = g->nx, ny = g->ny, nz = g->nz, d[3] = {nx, ny, nz};
    const uint64_t n = (uint64_t)nx * ny * nz;
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)n; ii++) {
        uint64_t i = (uint64_t)ii;
        b[i] = 0.0;
        if (cls[i] != 1) continue;
        uint32_t x = i % nx, y = (i / nx) % ny, z = (uint32_t)(i / ((uint64_t)nx * ny));
        double sum = 0.0;
        for (int a = 0; a < 3; a++) {
            int64_t l = nbr(d, g->periodic, x, y, z, a, -1), r = nbr(d, g->periodic, x, y, z, a, +1);
            uint32_t hx = x, hy = y, hz = z; /* canonical high face */
            double lo = 0.0, hi = 0.0;
            if (a == 0) {
                hx = (x + 1 == nx && (g->periodic & 1u)) ? 0 : x + 1;
                if (l >= 0 && cls[l] != 0) lo = u[x + (uint64_t)(nx + 1) * (y + (uint64_t)ny * z)];
                if (r >= 0 && cls[r] != 0) hi = u[hx + (uint64_t)(nx + 1) * (y + (uint64_t)ny * z)];
            } else if (a == 1) {
                hy = (y + 1 == ny && (g->periodic & 2u)) ? 0 : y + 1;
                if (l >= 0 && cls[l] != 0) lo = v[x + (uint64_t)nx * (y + (uint64_t)(ny + 1) * z)];
                if (r >= 0 && cls[r] != 0) hi = v[x + (uint64_t)nx * (hy + (uint64_t)(ny + 1) * z)];
            } else {
                hz = (z + 1 == nz && (g->periodic & 4u)) ? 0 : z + 1;
                if (l >= 0 && cls[l] != 0) lo = w[x + (uint64_t)nx * (y + (uint64_t)ny * z)];
                if ((r >= 0 && cls[r] != 0) || (outlet_on(g) && z + 1 == nz))
                    hi = w[x + (uint64_t)nx * (y + (uint64_t)ny * hz)];
            }
            sum += hi - lo;
        }
        b[i] = -(double)g->h * sum;
    }
}
static double *to_double(const float *a, uint64_t m) {
    double *d = (double *)malloc((m ? m : 1) * sizeof(double));
    for (uint64_t i = 0; i < m; i++) d[i] = a[i];
    return d;
}
static uint64_t nfaces(const onat_grid *g, int axis) {
    uint64_t nx = g->nx, ny = g->ny, nz = g->nz;
    return axis == 0 ? (nx + 1) * ny * nz : axis == 1 ? nx * (ny + 1) * nz : nx * ny * (nz + 1);
}
void onat_rhs(const onat_grid *g, const uint8_t *cls, const float *gtop, const float *u, const float *v,
              const float *w, double *b) {
    (void)gtop;
    double *ud = to_double(u, nfaces(g, 0)), *vd = to_double(v, nfaces(g, 1)), *wd = to_double(w, nfaces(g, 2));
    rhs_d(g, cls, ud, vd, wd, b);
    free(ud); free(vd); free(wd);
}
static inline double high_beta(const float *coef, const uint32_t *d, uint32_t periodic, uint32_t x, uint32_t y,
                               uint32_t z, int a) {
    int64_t r = nbr(d, periodic, x, y, z, a, +1);
    return r >= 0 ? (double)coef[4 * r + a] : 0.0;
}
static void apply_level(const uint32_t *d, uint32_t periodic, const float *coef, const double *x, double *y) {
    const uint64_t n = (uint64_t)d[0] * d[1] * d[2];
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)n; ii++) {
        uint64_t i = (uint64_t)ii;
        uint32_t cx = i % d[0], cy = (i / d[0]) % d[1], cz = (uint32_t)(i / ((uint64_t)d[0] * d[1]));
        double acc = (double)coef[4 * i + 3] * x[i];
        for (int a = 0; a < 3; a++) {
            double bl = coef[4 * i + a];
            if (bl != 0.0) acc += bl * (x[i] - x[nbr(d, periodic, cx, cy, cz, a, -1)]);
            double bh = high_beta(coef, d, periodic, cx, cy, cz, a);
            if (bh != 0.0) acc += bh * (x[i] - x[nbr(d, periodic, cx, cy, cz, a, +1)]);
        }
        y[i] = acc;
    }
}
void onat_apply(const onat_grid *g, const float *coef, const double *x, double *y) {
    const uint32_t d[3] = {g->nx, g->ny, g->nz};
    apply_level(d, g->periodic, coef, x, y);
}
static double diag_of(const float *coef, const uint32_t *d, uint32_t periodic, uint64_t i) {
    uint32_t x = i % d[0], y = (i / d[0]) % d[1], z = (uint32_t)(i / ((uint64_t)d[0] * d[1]));
    double s = coef[4 * i + 3];
    for (int a = 0; a < 3; a++) s += (double)coef[4 * i + a] + high_beta(coef, d, periodic, x, y, z, a);
    return s;
}

/* ------------------------------------------- aggregation V-cycle (FP64) */
typedef struct {
    uint32_t d[3];
    uint64_t n;
    float *coef;   /* (bx, by, bz, reaction) per cell, scaled by 4^-l */
    double *diag;
    double *r, *e, *tmp;
} mlevel;
typedef struct {
    int nl;
    uint32_t periodic;
    mlevel L[32];
    double *inv; /* dense inverse of the coarsest operator */
    double prolong;
} vcycle;

static void build_coarse(const mlevel *F, mlevel *C, uint32_t periodic) {
    for (int a = 0; a < 3; a++) C->d[a] = (F->d[a] + 1) / 2;
    C->n = (uint64_t)C->d[0] * C->d[1] * C->d[2];
    C->coef = (float *)calloc(4 * C->n, sizeof(float));
    for (uint64_t Q = 0; Q < C->n; Q++) {
        uint32_t qx = Q % C->d[0], qy = (Q / C->d[0]) % C->d[1], qz = (uint32_t)(Q / ((uint64_t)C->d[0] * C->d[1]));
        float c[4] = {0, 0, 0, 0};
        for (int z = 0; z < 2; z++)
            for (int y = 0; y < 2; y++)
                for (int x = 0; x < 2; x++) {
                    uint32_t cx = 2 * qx + x, cy = 2 * qy + y, cz = 2 * qz + z;
                    if (cx >= F->d[0] || cy >= F->d[1] || cz >= F->d[2]) continue;
                    uint64_t ci = cx + (uint64_t)F->d[0] * (cy + (uint64_t)F->d[1] * cz);
                    c[3] += F->coef[4 * ci + 3];
                    for (int a = 0; a < 3; a++) {
                        int64_t l = nbr(F->d, periodic, cx, cy, cz, a, -1);
                        if (l < 0) continue;
                        float beta = F->coef[4 * ci + a];
                        if (beta == 0.0f) continue;
                        uint32_t lx = l % F->d[0], ly = (l / F->d[0]) % F->d[1],
                                 lz = (uint32_t)(l / ((uint64_t)F->d[0] * F->d[1]));
                        if (lx / 2 == qx && ly / 2 == qy && lz / 2 == qz) continue;
                        c[a] += beta;
                    }
                }
        for (int k = 0; k < 4; k++) C->coef[4 * Q + k] = c[k] * 0.25f;
    }
}
static void level_alloc(mlevel *L, uint32_t periodic) {
    L->diag = (double *)malloc(L->n * sizeof(double));
    L->r = (double *)calloc(L->n, sizeof(double));
    L->e = (double *)calloc(L->n, sizeof(double));
    L->tmp = (double *)calloc(L->n, sizeof(double));
    for (uint64_t i = 0; i < L->n; i++) L->diag[i] = diag_of(L->coef, L->d, periodic, i);
}
/* Dense inverse by Gauss-Jordan with partial pivoting on rows with d > 0. */
static void coarse_inverse(vcycle *V) {
    mlevel *C = &V->L[V->nl - 1];
    uint64_t m = C->n;
    double *A = (double *)calloc(m * m, sizeof(double)), *I = (double *)calloc(m * m, sizeof(double));
    double *col = (double *)calloc(m, sizeof(double)), *out = (double *)calloc(m, sizeof(double));
    for (uint64_t k = 0; k < m; k++) {
        memset(col, 0, m * sizeof(double));
        col[k] = 1.0;
        apply_level(C->d, V->periodic, C->coef, col, out);
        for (uint64_t i = 0; i < m; i++) A[i * m + k] = out[i];
    }
    for (uint64_t i = 0; i < m; i++) {
        if (C->diag[i] <= 0.0) {
            for (uint64_t k = 0; k < m; k++) A[i * m + k] = A[k * m + i] = 0.0;
            A[i * m + i] = 1.0;
        }
        I[i * m + i] = 1.0;
    }
    for (uint64_t c = 0; c < m; c++) {
        uint64_t piv = c;
        for (uint64_t r = c + 1; r < m; r++)
            if (fabs(A[r * m + c]) > fabs(A[piv * m + c])) piv = r;
        if (piv != c)
            for (uint64_t k = 0; k < m; k++) {
                double t = A[c * m + k]; A[c * m + k] = A[piv * m + k]; A[piv * m + k] = t;
                t = I[c * m + k]; I[c * m + k] = I[piv * m + k]; I[piv * m + k] = t;
            }
        double p = A[c * m + c];
        if (fabs(p) < 1e-300) continue;
        for (uint64_t k = 0; k < m; k++) { A[c * m + k] /= p; I[c * m + k] /= p; }
        for (uint64_t r = 0; r < m; r++) {
            if (r == c) continue;
            double f = A[r * m + c];
            if (f == 0.0) continue;
            for (uint64_t k = 0; k < m; k++) { A[r * m + k] -= f * A[c * m + k]; I[r * m + k] -= f * I[c * m + k]; }
        }
    }
    V->inv = (double *)calloc(m * m, sizeof(double));
    for (uint64_t i = 0; i < m; i++)
        for (uint64_t k = 0; k < m; k++)
            V->inv[i * m + k] = (C->diag[i] > 0.0 && C->diag[k] > 0.0) ? 0.5 * (I[i * m + k] + I[k * m + i]) : 0.0;
    free(A); free(I); free(col); free(out);
}
static vcycle *vcycle_new(const uint32_t *d, uint32_t periodic, const float *coef, double prolong) {
    vcycle *V = (vcycle *)calloc(1, sizeof *V);
    V->periodic = periodic;
    V->prolong = prolong;
    mlevel *F = &V->L[0];
    memcpy(F->d, d, sizeof F->d);
    F->n = (uint64_t)d[0] * d[1] * d[2];
    F->coef = (float *)malloc(4 * F->n * sizeof(float));
    memcpy(F->coef, coef, 4 * F->n * sizeof(float));
    level_alloc(F, periodic);
    V->nl = 1;
    while (V->L[V->nl - 1].d[0] > 4 || V->L[V->nl - 1].d[1] > 4 || V->L[V->nl - 1].d[2] > 4) {
        build_coarse(&V->L[V->nl - 1], &V->L[V->nl], periodic);
        level_alloc(&V->L[V->nl], periodic);
        V->nl++;
    }
    coarse_inverse(V);
    return V;
}
static void vcycle_free(vcycle *V) {
    for (int l = 0; l < V->nl; l++) {
        free(V->L[l].coef); free(V->L[l].diag); free(V->L[l].r); free(V->L[l].e); free(V->L[l].tmp);
    }
    free(V->inv);
    free(V);
}
/* One half-step of red-black Gauss-Seidel: every cell of `color` is updated
 * from the values at the start of the half-step (the GPU's semantics). */
static void rb_half(const mlevel *L, uint32_t periodic, int color) {
    const uint32_t *d = L->d;
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)L->n; ii++) {
        uint64_t i = (uint64_t)ii;
        uint32_t x = i % d[0], y = (i / d[0]) % d[1], z = (uint32_t)(i / ((uint64_t)d[0] * d[1]));
        if (((x + y + z) & 1u) != (uint32_t)color) continue;
        if (L->diag[i] <= 0.0) { L->tmp[i] = 0.0; continue; }
        double s = L->r[i];
        for (int a = 0; a < 3; a++) {
            double bl = L->coef[4 * i + a];
            if (bl != 0.0) s += bl * L->e[nbr(d, periodic, x, y, z, a, -1)];
            double bh = high_beta(L->coef, d, periodic, x, y, z, a);
            if (bh != 0.0) s += bh * L->e[nbr(d, periodic, x, y, z, a, +1)];
        }
        L->tmp[i] = s / L->diag[i];
    }
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)L->n; ii++) {
        uint64_t i = (uint64_t)ii;
        uint32_t x = i % d[0], y = (i / d[0]) % d[1], z = (uint32_t)(i / ((uint64_t)d[0] * d[1]));
        if (((x + y + z) & 1u) == (uint32_t)color) L->e[i] = L->tmp[i];
    }
}
static void vcycle_level(vcycle *V, int l) {
    mlevel *L = &V->L[l];
    if (l == V->nl - 1) {
        for (uint64_t i = 0; i < L->n; i++) {
            double s = 0.0;
            for (uint64_t k = 0; k < L->n; k++) s += V->inv[i * L->n + k] * L->r[k];
            L->e[i] = s;
        }
        return;
    }
    memset(L->e, 0, L->n * sizeof(double));
    rb_half(L, V->periodic, 0);
    rb_half(L, V->periodic, 1);
    /* residual and restriction: r_{l+1} = 1/4 * sum over the 8 children */
    mlevel *C = &V->L[l + 1];
    apply_level(L->d, V->periodic, L->coef, L->e, L->tmp);
    memset(C->r, 0, C->n * sizeof(double));
    for (uint64_t i = 0; i < L->n; i++) {
        uint32_t x = i % L->d[0], y = (i / L->d[0]) % L->d[1], z = (uint32_t)(i / ((uint64_t)L->d[0] * L->d[1]));
        uint64_t Q = x / 2 + (uint64_t)C->d[0] * (y / 2 + (uint64_t)C->d[1] * (z / 2));
        C->r[Q] += L->r[i] - L->tmp[i];
    }
    for (uint64_t Q = 0; Q < C->n; Q++) C->r[Q] *= 0.25;
    vcycle_level(V, l + 1);
    for (uint64_t i = 0; i < L->n; i++) {
        if (L->diag[i] <= 0.0) continue;
        uint32_t x = i % L->d[0], y = (i / L->d[0]) % L->d[1], z = (uint32_t)(i / ((uint64_t)L->d[0] * L->d[1]));
        L->e[i] += V->prolong * C->e[x / 2 + (uint64_t)C->d[0] * (y / 2 + (uint64_t)C->d[1] * (z / 2))];
    }
    rb_half(L, V->periodic, 1);
    rb_half(L, V->periodic, 0);
}
static void vcycle_apply(vcycle *V, const double *r, double *z) {
    memcpy(V->L[0].r, r, V->L[0].n * sizeof(double));
    vcycle_level(V, 0);
    memcpy(z, V->L[0].e, V->L[0].n * sizeof(double));
}

/* Coarse-correction weight of the V-cycle (the GPU path's default is 2). */
static double g_prolong = 2.0;
void onat_set_prolongation(double w) { g_prolong = w; }

/* ---------------------------------------------------------------- PCG */
static double dot(const double *a, const double *b, uint64_t n) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) s += a[i] * b[i];
    return s;
}
int onat_solve(const onat_grid *g, const float *coef, const uint8_t *cls, const double *b, double *x, double rtol,
               int max_it, int *iterations, double *rel_residual) {
    const uint32_t d[3] = {g->nx, g->ny, g->nz};
    const uint64_t n = (uint64_t)g->nx * g->ny * g->nz;
    double *r = (double *)malloc(n * sizeof(double)), *z = (double *)malloc(n * sizeof(double));
    double *p = (double *)malloc(n * sizeof(double)), *q = (double *)malloc(n * sizeof(double));
    vcycle *V = vcycle_new(d, g->periodic, coef, g_prolong);
    double bb = sqrt(dot(b, b, n));
    int it = 0, status = 1;
    double rel = 0.0;
    for (uint64_t i = 0; i < n; i++)
        if (cls[i] != 1) x[i] = 0.0;
    if (bb == 0.0) {
        memset(x, 0, n * sizeof(double));
        status = 0;
        goto done;
    }
    for (int restart = 0; restart < 8 && it < max_it; restart++) {
        apply_level(d, g->periodic, coef, x, q);
        for (uint64_t i = 0; i < n; i++) r[i] = cls[i] == 1 ? b[i] - q[i] : 0.0;
        rel = sqrt(dot(r, r, n)) / bb;
        if (rel <= rtol) { status = 0; break; }
        vcycle_apply(V, r, z);
        memcpy(p, z, n * sizeof(double));
        double rz = dot(r, z, n);
        while (it < max_it) {
            apply_level(d, g->periodic, coef, p, q);
            double alpha = rz / dot(p, q, n);
            for (uint64_t i = 0; i < n; i++) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
            it++;
            if (sqrt(dot(r, r, n)) <= 0.5 * rtol * bb) break;
            vcycle_apply(V, r, z);
            double rz1 = dot(r, z, n), beta = rz1 / rz;
            rz = rz1;
            for (uint64_t i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
        }
    }
    apply_level(d, g->periodic, coef, x, q);
    for (uint64_t i = 0; i < n; i++) r[i] = cls[i] == 1 ? b[i] - q[i] : 0.0;
    rel = sqrt(dot(r, r, n)) / bb;
    if (rel <= rtol) status = 0;
done:
    if (iterations) *iterations = it;
    if (rel_residual) *rel_residual = rel;
    vcycle_free(V);
    free(r); free(z); free(p); free(q);
    return status;
}

/* ------------------------------------------------------ correction */
static void correct_d(const onat_grid *g, const float *alpha, const uint8_t *cls, const float *gtop, const double *phi,
                      const double *us, const double *vs, const double *ws, double *u, double *v, double *w) {
    const uint32_t nx = g->nx, ny = g->ny, nz = g->nz;
    const double h = g->h;
    /* x faces: (nx+1) x ny x nz */
#pragma omp parallel for schedule(static)
    for (int64_t zz = 0; zz < (int64_t)nz; zz++)
        for (uint32_t y = 0; y < ny; y++)
            for (uint32_t x = 0; x <= nx; x++) {
                uint32_t z = (uint32_t)zz;
                uint64_t f = x + (uint64_t)(nx + 1) * (y + (uint64_t)ny * z);
                double out = 0.0;
                int has = 1;
                uint32_t xl = x - 1, xr = x;
                if (x == 0 || x == nx) {
                    if (g->periodic & 1u) { xl = nx - 1; xr = 0; }
                    else has = 0;
                }
                if (has) {
                    uint64_t L = xl + (uint64_t)nx * (y + (uint64_t)ny * z), R = xr + (uint64_t)nx * (y + (uint64_t)ny * z);
                    if (cls[L] != 0 && cls[R] != 0) {
                        uint64_t fc = xr + (uint64_t)(nx + 1) * (y + (uint64_t)ny * z);
                        out = (double)us[fc] - (double)nbeta(g, alpha, L, R) * (phi[R] - phi[L]) / h;
                    }
                }
                u[f] = out;
            }
#pragma omp parallel for schedule(static)
    for (int64_t zz = 0; zz < (int64_t)nz; zz++)
        for (uint32_t y = 0; y <= ny; y++)
            for (uint32_t x = 0; x < nx; x++) {
                uint32_t z = (uint32_t)zz;
                uint64_t f = x + (uint64_t)nx * (y + (uint64_t)(ny + 1) * z);
                double out = 0.0;
                int has = 1;
                uint32_t yl = y - 1, yr = y;
                if (y == 0 || y == ny) {
                    if (g->periodic & 2u) { yl = ny - 1; yr = 0; }
                    else has = 0;
                }
                if (has) {
                    uint64_t L = x + (uint64_t)nx * (yl + (uint64_t)ny * z), R = x + (uint64_t)nx * (yr + (uint64_t)ny * z);
                    if (cls[L] != 0 && cls[R] != 0) {
                        uint64_t fc = x + (uint64_t)nx * (yr + (uint64_t)(ny + 1) * z);
                        out = (double)vs[fc] - (double)nbeta(g, alpha, L, R) * (phi[R] - phi[L]) / h;
                    }
                }
                v[f] = out;
            }
#pragma omp parallel for schedule(static)
    for (int64_t zz = 0; zz <= (int64_t)nz; zz++)
        for (uint32_t y = 0; y < ny; y++)
            for (uint32_t x = 0; x < nx; x++) {
                uint32_t z = (uint32_t)zz;
                uint64_t f = x + (uint64_t)nx * (y + (uint64_t)ny * z);
                double out = 0.0;
                if (z == nz && outlet_on(g)) {
                    uint64_t C = x + (uint64_t)nx * (y + (uint64_t)ny * (nz - 1));
                    if (cls[C] != 0) out = (double)ws[f] + (double)gtop[x + (uint64_t)nx * y] * phi[C] / h;
                } else {
                    int has = 1;
                    uint32_t zl = z - 1, zr = z;
                    if (z == 0 || z == nz) {
                        if (g->periodic & 4u) { zl = nz - 1; zr = 0; }
                        else has = 0;
                    }
                    if (has) {
                        uint64_t L = x + (uint64_t)nx * (y + (uint64_t)ny * zl), R = x + (uint64_t)nx * (y + (uint64_t)ny * zr);
                        if (cls[L] != 0 && cls[R] != 0) {
                            uint64_t fc = x + (uint64_t)nx * (y + (uint64_t)ny * zr);
                            out = (double)ws[fc] - (double)nbeta(g, alpha, L, R) * (phi[R] - phi[L]) / h;
                        }
                    }
                }
                w[f] = out;
            }
}

void onat_correct(const onat_grid *g, const float *alpha, const uint8_t *cls, const float *gtop, const double *phi,
                  const float *us, const float *vs, const float *ws, double *u, double *v, double *w) {
    double *ud = to_double(us, nfaces(g, 0)), *vd = to_double(vs, nfaces(g, 1)), *wd = to_double(ws, nfaces(g, 2));
    correct_d(g, alpha, cls, gtop, phi, ud, vd, wd, u, v, w);
    free(ud); free(vd); free(wd);
}

void onat_divergence(const onat_grid *g, const uint8_t *cls, const float *gtop, const double *u, const double *v,
                     const double *w, double *max_abs, double *rms) {
    (void)gtop;
    const uint32_t nx = g->nx, ny = g->ny, nz = g->nz;
    double mx = 0.0, ss = 0.0;
    uint64_t count = 0;
    for (uint32_t z = 0; z < nz; z++)
        for (uint32_t y = 0; y < ny; y++)
            for (uint32_t x = 0; x < nx; x++) {
                uint64_t i = x + (uint64_t)nx * (y + (uint64_t)ny * z);
                if (cls[i] != 1) continue;
                double dv = u[x + 1 + (uint64_t)(nx + 1) * (y + (uint64_t)ny * z)] - u[x + (uint64_t)(nx + 1) * (y + (uint64_t)ny * z)];
                dv += v[x + (uint64_t)nx * (y + 1 + (uint64_t)(ny + 1) * z)] - v[x + (uint64_t)nx * (y + (uint64_t)(ny + 1) * z)];
                dv += w[x + (uint64_t)nx * (y + (uint64_t)ny * (z + 1))] - w[x + (uint64_t)nx * (y + (uint64_t)ny * z)];
                dv /= g->h;
                if (fabs(dv) > mx) mx = fabs(dv);
                ss += dv * dv;
                count++;
            }
    *max_abs = mx;
    *rms = count ? sqrt(ss / count) : 0.0;
}

/* --------------------------------------------------------- projection */
typedef struct {
    uint64_t n;
    uint8_t *cls;
    float *coef, *gtop;
} prepared;
static void prepare(const onat_grid *g, const float *alpha, const uint8_t *solid, prepared *P) {
    P->n = (uint64_t)g->nx * g->ny * g->nz;
    P->cls = (uint8_t *)malloc(P->n);
    P->coef = (float *)malloc(4 * P->n * sizeof(float));
    P->gtop = (float *)malloc((uint64_t)g->nx * g->ny * sizeof(float));
    onat_classify(g, solid, P->cls);
    onat_coefficients(g, alpha, P->cls, P->coef, P->gtop);
}
static void release(prepared *P) { free(P->cls); free(P->coef); free(P->gtop); }

static int project_d(const onat_grid *g, const float *alpha, const uint8_t *solid, const double *us, const double *vs,
                     const double *ws, float dt, double rtol, double *phi, double *u, double *v, double *w, double *p,
                     int *iterations, double *rel_residual) {
    prepared P;
    prepare(g, alpha, solid, &P);
    double *b = (double *)malloc(P.n * sizeof(double));
    rhs_d(g, P.cls, us, vs, ws, b);
    memset(phi, 0, P.n * sizeof(double));
    int st = onat_solve(g, P.coef, P.cls, b, phi, rtol, 100000, iterations, rel_residual);
    correct_d(g, alpha, P.cls, P.gtop, phi, us, vs, ws, u, v, w);
    if (p)
        for (uint64_t i = 0; i < P.n; i++) p[i] = P.cls[i] ? (double)g->rho_liquid * phi[i] / (double)dt : 0.0;
    free(b);
    release(&P);
    return st;
}

int onat_project(const onat_grid *g, const float *alpha, const uint8_t *solid, const float *us, const float *vs,
                 const float *ws, float dt, double rtol, double *phi, double *u, double *v, double *w, double *p,
                 int *iterations, double *rel_residual) {
    double *ud = to_double(us, nfaces(g, 0)), *vd = to_double(vs, nfaces(g, 1)), *wd = to_double(ws, nfaces(g, 2));
    int st = project_d(g, alpha, solid, ud, vd, wd, dt, rtol, phi, u, v, w, p, iterations, rel_residual);
    free(ud); free(vd); free(wd);
    return st;
}

/* ------------------------------------------------------------ adjoint */
/* Face loops shared by the adjoint: for every open face call fn with the
 * canonical face index, the two cells (R = -1 for an outlet face) and beta
 * (or the outlet conductance). */
typedef struct { uint64_t fc; int64_t L, R; double beta; int duplicate; uint64_t f; } oface;
static uint64_t faces_of(const onat_grid *g, int axis) {
    uint64_t nx = g->nx, ny = g->ny, nz = g->nz;
    if (axis == 0) return (nx + 1) * ny * nz;
    if (axis == 1) return nx * (ny + 1) * nz;
    return nx * ny * (nz + 1);
}
static int face_info(const onat_grid *g, const float *alpha, const uint8_t *cls, const float *gtop, int axis,
                     uint64_t f, oface *o) {
    uint64_t nx = g->nx, ny = g->ny, nz = g->nz;
    uint64_t D[3] = {nx, ny, nz}, F[3] = {nx, ny, nz};
    F[axis] += 1;
    uint64_t c[3] = {f % F[0], (f / F[0]) % F[1], f / (F[0] * F[1])};
    o->f = f;
    o->duplicate = 0;
    uint64_t lo[3] = {c[0], c[1], c[2]}, hi[3] = {c[0], c[1], c[2]};
    if (c[axis] == 0 || c[axis] == D[axis]) {
        if (g->periodic & (1u << axis)) {
            o->duplicate = c[axis] == D[axis];
            lo[axis] = D[axis] - 1;
            hi[axis] = 0;
        } else if (axis == 2 && c[2] == nz && outlet_on(g)) {
            uint64_t C = c[0] + nx * (c[1] + ny * (nz - 1));
            if (cls[C] == 0) return 0;
            o->fc = f;
            o->L = (int64_t)C;
            o->R = -1;
            o->beta = gtop[c[0] + nx * c[1]];
            return 1;
        } else {
            return 0;
        }
    } else {
        lo[axis] = c[axis] - 1;
    }
    uint64_t L = lo[0] + nx * (lo[1] + ny * lo[2]), R = hi[0] + nx * (hi[1] + ny * hi[2]);
    if (cls[L] == 0 || cls[R] == 0) return 0;
    uint64_t cc[3] = {hi[0], hi[1], hi[2]};
    o->fc = cc[0] + F[0] * (cc[1] + F[1] * cc[2]);
    o->L = (int64_t)L;
    o->R = (int64_t)R;
    o->beta = nbeta(g, alpha, L, R);
    return 1;
}

int onat_project_vjp(const onat_grid *g, const float *alpha, const uint8_t *solid, const double *gu, const double *gv,
                     const double *gw, const double *gp, float dt, double rtol, double *gus, double *gvs,
                     double *gws) {
    prepared P;
    prepare(g, alpha, solid, &P);
    const double h = g->h;
    const double *gin[3] = {gu, gv, gw};
    double *gout[3] = {gus, gvs, gws};
    double *gphi = (double *)calloc(P.n, sizeof(double)), *gb = (double *)calloc(P.n, sizeof(double));
    double *fold[3];
    /* Fold the gradient of periodic duplicate faces into the canonical face. */
    for (int a = 0; a < 3; a++) {
        uint64_t m = faces_of(g, a);
        fold[a] = (double *)malloc(m * sizeof(double));
        memcpy(fold[a], gin[a], m * sizeof(double));
        for (uint64_t f = 0; f < m; f++) {
            oface o;
            if (face_info(g, alpha, P.cls, P.gtop, a, f, &o) && o.duplicate) {
                fold[a][o.fc] += gin[a][f];
                fold[a][f] = 0.0;
            }
        }
    }
    /* gphi = d u / d phi ^T g_u + rho_l/dt g_p on active cells */
    for (int a = 0; a < 3; a++) {
        uint64_t m = faces_of(g, a);
        for (uint64_t f = 0; f < m; f++) {
            oface o;
            if (!face_info(g, alpha, P.cls, P.gtop, a, f, &o) || o.duplicate) continue;
            double gf = fold[a][o.fc];
            if (o.R < 0) {
                if (P.cls[o.L] == 1) gphi[o.L] += o.beta / h * gf;
            } else {
                if (P.cls[o.R] == 1) gphi[o.R] -= o.beta / h * gf;
                if (P.cls[o.L] == 1) gphi[o.L] += o.beta / h * gf;
            }
        }
    }
    if (gp)
        for (uint64_t i = 0; i < P.n; i++)
            if (P.cls[i] == 1) gphi[i] += (double)g->rho_liquid / (double)dt * gp[i];
    int it;
    double rel;
    int st = onat_solve(g, P.coef, P.cls, gphi, gb, rtol, 100000, &it, &rel);
    for (int a = 0; a < 3; a++) {
        uint64_t m = faces_of(g, a);
        for (uint64_t f = 0; f < m; f++) gout[a][f] = 0.0;
        for (uint64_t f = 0; f < m; f++) {
            oface o;
            if (!face_info(g, alpha, P.cls, P.gtop, a, f, &o) || o.duplicate) continue;
            double acc = fold[a][o.fc];
            if (o.R < 0) {
                if (P.cls[o.L] == 1) acc += -h * gb[o.L];
            } else {
                if (P.cls[o.L] == 1) acc += -h * gb[o.L];
                if (P.cls[o.R] == 1) acc -= -h * gb[o.R];
            }
            gout[a][o.fc] = acc;
        }
        free(fold[a]);
    }
    free(gphi);
    free(gb);
    release(&P);
    return st;
}

/* ---------------------------------------------------------------- chain */
static double face_density_of(const onat_grid *g, const float *alpha, const oface *o) {
    if (o->R < 0) return nrho(g, alpha[o->L]);
    return 0.5 * ((double)nrho(g, alpha[o->L]) + (double)nrho(g, alpha[o->R]));
}
int onat_chain_forward(const onat_grid *g, const float *alpha, const uint8_t *solid, const float *u0, const float *v0,
                       const float *w0, const float *fu, const float *fv, const float *fw, float dt, int steps,
                       double rtol, double *uk, double *vk, double *wk, double *objective) {
    /* States stay in FP64 between steps: the oracle's chain has no FP32 rounding. */
    const uint64_t m[3] = {faces_of(g, 0), faces_of(g, 1), faces_of(g, 2)};
    const uint64_t n = (uint64_t)g->nx * g->ny * g->nz;
    prepared P;
    prepare(g, alpha, solid, &P);
    double *cur[3], *star[3];
    const float *init[3] = {u0, v0, w0}, *force[3] = {fu, fv, fw};
    double *out[3] = {uk, vk, wk};
    for (int a = 0; a < 3; a++) {
        cur[a] = to_double(init[a], m[a]);
        star[a] = (double *)malloc(m[a] * sizeof(double));
    }
    double *phi = (double *)malloc(n * sizeof(double));
    int st = 0;
    for (int k = 0; k < steps; k++) {
        for (int a = 0; a < 3; a++) {
            memcpy(star[a], cur[a], m[a] * sizeof(double));
            for (uint64_t f = 0; f < m[a]; f++) {
                oface o;
                if (!face_info(g, alpha, P.cls, P.gtop, a, f, &o) || o.duplicate) continue;
                star[a][o.fc] = cur[a][o.fc] + (double)dt * (double)force[a][o.fc] / face_density_of(g, alpha, &o);
            }
        }
        int it;
        double rel;
        st |= project_d(g, alpha, solid, star[0], star[1], star[2], dt, rtol, phi, cur[0], cur[1], cur[2], NULL, &it,
                        &rel);
    }
    double J = 0.0;
    for (int a = 0; a < 3; a++) memcpy(out[a], cur[a], m[a] * sizeof(double));
    if (outlet_on(g))
        for (uint64_t y = 0; y < g->ny; y++)
            for (uint64_t x = 0; x < g->nx; x++) {
                double wz = cur[2][x + (uint64_t)g->nx * (y + (uint64_t)g->ny * g->nz)];
                J += wz * wz;
            }
    *objective = J;
    for (int a = 0; a < 3; a++) { free(cur[a]); free(star[a]); }
    free(phi);
    release(&P);
    return st;
}
int onat_chain_adjoint(const onat_grid *g, const float *alpha, const uint8_t *solid, const double *uk,
                       const double *vk, const double *wk, float dt, int steps, double rtol, double *gfu,
                       double *gfv, double *gfw) {
    (void)uk; (void)vk;
    const uint64_t m[3] = {faces_of(g, 0), faces_of(g, 1), faces_of(g, 2)};
    prepared P;
    prepare(g, alpha, solid, &P);
    double *lam[3], *nxt[3], *gf[3] = {gfu, gfv, gfw};
    for (int a = 0; a < 3; a++) {
        lam[a] = (double *)calloc(m[a], sizeof(double));
        nxt[a] = (double *)calloc(m[a], sizeof(double));
        memset(gf[a], 0, m[a] * sizeof(double));
    }
    if (outlet_on(g))
        for (uint64_t y = 0; y < g->ny; y++)
            for (uint64_t x = 0; x < g->nx; x++) {
                uint64_t f = x + (uint64_t)g->nx * (y + (uint64_t)g->ny * g->nz);
                lam[2][f] = 2.0 * wk[f];
            }
    int st = 0;
    for (int k = steps - 1; k >= 0; k--) {
        st |= onat_project_vjp(g, alpha, solid, lam[0], lam[1], lam[2], NULL, dt, rtol, nxt[0], nxt[1], nxt[2]);
        for (int a = 0; a < 3; a++) {
            memcpy(lam[a], nxt[a], m[a] * sizeof(double));
            for (uint64_t f = 0; f < m[a]; f++) {
                oface o;
                if (!face_info(g, alpha, P.cls, P.gtop, a, f, &o) || o.duplicate) continue;
                gf[a][o.fc] += (double)dt / face_density_of(g, alpha, &o) * lam[a][o.fc];
            }
        }
    }
    for (int a = 0; a < 3; a++) { free(lam[a]); free(nxt[a]); }
    release(&P);
    return st;
}

/* Summed outlet objective: every state after a step contributes, so the
 * adjoint of step k adds 2 w_k on the outlet faces to lambda before the VJP
 * of step k-1.  Test oracle for the GPU chain's checkpoint recompute. */
int onat_chain_summed(const onat_grid *g, const float *alpha, const uint8_t *solid, const float *u0,
                      const float *v0, const float *w0, const float *fu, const float *fv, const float *fw, float dt,
                      int steps, double rtol, double *objective, double *gfu, double *gfv, double *gfw) {
    const uint64_t m[3] = {faces_of(g, 0), faces_of(g, 1), faces_of(g, 2)};
    const uint64_t n = (uint64_t)g->nx * g->ny * g->nz;
    const uint64_t top = (uint64_t)g->nx * g->ny * g->nz;  /* first outlet w face */
    const uint64_t plane = (uint64_t)g->nx * g->ny;
    prepared P;
    prepare(g, alpha, solid, &P);
    /* states[k][a]: u_k, k = 0 .. steps */
    double **states = (double **)malloc((size_t)(steps + 1) * 3 * sizeof(double *));
    const float *init[3] = {u0, v0, w0}, *force[3] = {fu, fv, fw};
    double *star[3];
    for (int a = 0; a < 3; a++) {
        states[a] = to_double(init[a], m[a]);
        star[a] = (double *)malloc(m[a] * sizeof(double));
    }
    double *phi = (double *)malloc(n * sizeof(double));
    int st = 0;
    double J = 0.0;
    for (int k = 0; k < steps; k++) {
        double **cur = states + 3 * k, **nx_ = states + 3 * (k + 1);
        for (int a = 0; a < 3; a++) {
            nx_[a] = (double *)malloc(m[a] * sizeof(double));
            memcpy(star[a], cur[a], m[a] * sizeof(double));
            for (uint64_t f = 0; f < m[a]; f++) {
                oface o;
                if (!face_info(g, alpha, P.cls, P.gtop, a, f, &o) || o.duplicate) continue;
                star[a][o.fc] = cur[a][o.fc] + (double)dt * (double)force[a][o.fc] / face_density_of(g, alpha, &o);
            }
        }
        int it;
        double rel;
        st |= project_d(g, alpha, solid, star[0], star[1], star[2], dt, rtol, phi, nx_[0], nx_[1], nx_[2], NULL, &it,
                        &rel);
        if (outlet_on(g))
            for (uint64_t f = 0; f < plane; f++) J += nx_[2][top + f] * nx_[2][top + f];
    }
    *objective = J;
    if (gfu && gfv && gfw) {
        double *lam[3], *nxt[3], *gf[3] = {gfu, gfv, gfw};
        for (int a = 0; a < 3; a++) {
            lam[a] = (double *)calloc(m[a], sizeof(double));
            nxt[a] = (double *)calloc(m[a], sizeof(double));
            memset(gf[a], 0, m[a] * sizeof(double));
        }
        if (outlet_on(g))
            for (uint64_t f = 0; f < plane; f++) lam[2][top + f] = 2.0 * states[3 * steps + 2][top + f];
        for (int k = steps - 1; k >= 0; k--) {
            st |= onat_project_vjp(g, alpha, solid, lam[0], lam[1], lam[2], NULL, dt, rtol, nxt[0], nxt[1], nxt[2]);
            for (int a = 0; a < 3; a++) {
                memcpy(lam[a], nxt[a], m[a] * sizeof(double));
                for (uint64_t f = 0; f < m[a]; f++) {
                    oface o;
                    if (!face_info(g, alpha, P.cls, P.gtop, a, f, &o) || o.duplicate) continue;
                    gf[a][o.fc] += (double)dt / face_density_of(g, alpha, &o) * lam[a][o.fc];
                }
            }
            if (k >= 1 && outlet_on(g))
                for (uint64_t f = 0; f < plane; f++) lam[2][top + f] += 2.0 * states[3 * k + 2][top + f];
        }
        for (int a = 0; a < 3; a++) { free(lam[a]); free(nxt[a]); }
    }
    for (int k = 0; k <= steps; k++)
        for (int a = 0; a < 3; a++) free(states[3 * k + a]);
    free(states);
    for (int a = 0; a < 3; a++) free(star[a]);
    free(phi);
    release(&P);
    return st;
}
