/*
 * ifl_oracle.c - CPU oracle (plain C) for the incremental-fluids hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker for the CUDA path and the timed
 * CPU baseline in bench.py.  Never part of the product path.
 *
 * A restatement, in this project's own C, of FluidSolver::update from the
 * reference tutorial steps 1-8 (tunabrain/incremental-fluids).  Each function
 * cites the reference lines whose arithmetic it follows.  The floating-point
 * operation order of every cell update is kept identical to the reference so
 * that results are bit-identical when both sides are compiled with
 * -ffp-contract=off; this is checked against the reference's own sources in
 * tests/test_oracle_pin.py.
 *
 * Differences from the reference, all deliberate and documented:
 *  - every buffer is zero-initialised (the reference reads uninitialised
 *    `new double[]` memory in its solid variants);
 *  - the reference's out-of-range accesses (addInflow's x bound uses the
 *    grid height, step 7 indexes v-face densities with the u-grid width, the
 *    extrapolation stack can reach the outer ring) are reproduced as flat-index
 *    arithmetic where they stay inside the array and skipped where they leave
 *    it; the GPU path reproduces the same flat-index behaviour;
 *  - nothing is printed (the reference printf's the PCG outcome; the oracle
 *    records it in ifo_pcg_stats instead).
 */
#include "ifl_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define CELL_FLUID 0
#define CELL_SOLID 1
#define CELL_EMPTY 2
#define PCG_TOL 1e-5
#define MIC_TAU 0.97
#define MIC_SIGMA 0.25

/* std::min / std::max semantics: min(a,b) = (b < a) ? b : a,
 * max(a,b) = (a < b) ? b : a.  NaN handling follows from these forms. */
static inline double smin(double a, double b) { return (b < a) ? b : a; }
static inline double smax(double a, double b) { return (a < b) ? b : a; }
static inline int imin(int a, int b) { return (b < a) ? b : a; }
static inline int imax(int a, int b) { return (a < b) ? b : a; }
/* sgn / nsgn: 4-solid-boundaries/Fluid.cpp:38-45 */
static inline int sgn(double v) { return (0.0 < v) - (v < 0.0); }
static inline int nsgn(double v) { return v < 0.0 ? -1 : 1; }

/* 3-conjugate-gradients/Fluid.cpp:32-39 */
static double length2(double x, double y) { return sqrt(x * x + y * y); }
static double cubic_pulse(double x) {
    x = smin(fabs(x), 1.0);
    return 1.0 - x * x * (3.0 - 2.0 * x);
}

/* 4-solid-boundaries/Fluid.cpp:58-62 (trig evaluated at every call) */
static void rotate(double *x, double *y, double phi) {
    double tx = *x, ty = *y;
    *x = cos(phi) * tx + sin(phi) * ty;
    *y = -sin(phi) * tx + cos(phi) * ty;
}

/* ---------------------------------------------------------------- bodies */

/* SolidBox::distance 4-solid-boundaries/Fluid.cpp:158-169,
 * SolidSphere::distance :210-212 */
static double body_distance(const ifo_body *b, double x, double y) {
    if (b->type == 0) {
        x -= b->pos_x;
        y -= b->pos_y;
        rotate(&x, &y, -b->theta);
        double dx = fabs(x) - b->scale_x * 0.5;
        double dy = fabs(y) - b->scale_y * 0.5;
        if (dx >= 0.0 || dy >= 0.0)
            return length2(smax(dx, 0.0), smax(dy, 0.0));
        return smax(dx, dy);
    }
    return length2(x - b->pos_x, y - b->pos_y) - b->scale_x * 0.5;
}

/* SolidBox::closestSurfacePoint :171-186, SolidSphere :214-227 with
 * globalToLocal / localToGlobal :92-107 */
static void body_closest(const ifo_body *b, double *px, double *py) {
    double x = *px, y = *py;
    if (b->type == 0) {
        x -= b->pos_x;
        y -= b->pos_y;
        rotate(&x, &y, -b->theta);
        double dx = fabs(x) - b->scale_x * 0.5;
        double dy = fabs(y) - b->scale_y * 0.5;
        if (dx > dy)
            x = nsgn(x) * 0.5 * b->scale_x;
        else
            y = nsgn(y) * 0.5 * b->scale_y;
        rotate(&x, &y, b->theta);
        x += b->pos_x;
        y += b->pos_y;
    } else {
        x -= b->pos_x;
        y -= b->pos_y;
        rotate(&x, &y, -b->theta);
        x /= b->scale_x;
        y /= b->scale_y;
        double r = length2(x, y);
        if (r < 1e-4) {
            x = 0.5;
            y = 0.0;
        } else {
            x /= 2.0 * r;
            y /= 2.0 * r;
        }
        x *= b->scale_x;
        y *= b->scale_y;
        rotate(&x, &y, b->theta);
        x += b->pos_x;
        y += b->pos_y;
    }
    *px = x;
    *py = y;
}

/* SolidBox::distanceNormal :188-200, SolidSphere::distanceNormal :229-240
 * (the sphere rounds its radius through float) */
static void body_normal(const ifo_body *b, double *nx, double *ny, double x, double y) {
    if (b->type == 0) {
        x -= b->pos_x;
        y -= b->pos_y;
        rotate(&x, &y, -b->theta);
        if (fabs(x) - b->scale_x * 0.5 > fabs(y) - b->scale_y * 0.5) {
            *nx = nsgn(x);
            *ny = 0.0;
        } else {
            *nx = 0.0;
            *ny = nsgn(y);
        }
        rotate(nx, ny, b->theta);
    } else {
        x -= b->pos_x;
        y -= b->pos_y;
        float r = (float)length2(x, y);
        if (r < 1e-4) {
            *nx = 1.0;
            *ny = 0.0;
        } else {
            *nx = x / r;
            *ny = y / r;
        }
    }
}

/* SolidBody::velocityX/Y :127-133 */
static double body_vel_x(const ifo_body *b, double x, double y) {
    (void)x;
    return (b->pos_y - y) * b->vel_theta + b->vel_x;
}
static double body_vel_y(const ifo_body *b, double x, double y) {
    (void)y;
    return (x - b->pos_x) * b->vel_theta + b->vel_y;
}

/* occupancy: 7-variable-density/Fluid.cpp:60-102 */
static double tri_occ(double out1, double in, double out2) {
    return 0.5 * in * in / ((out1 - in) * (out2 - in));
}
static double trap_occ(double out1, double out2, double in1, double in2) {
    return 0.5 * (-in1 / (out1 - in1) - in2 / (out2 - in2));
}
static double occupancy(double d11, double d12, double d21, double d22) {
    double ds[4] = {d11, d12, d22, d21};
    uint8_t b = 0;
    for (int i = 3; i >= 0; i--)
        b = (uint8_t)((b << 1) | (ds[i] < 0.0 ? 1 : 0));
    switch (b) {
    case 0x0: return 0.0;
    case 0x1: return tri_occ(d21, d11, d12);
    case 0x2: return tri_occ(d11, d12, d22);
    case 0x4: return tri_occ(d12, d22, d21);
    case 0x8: return tri_occ(d22, d21, d11);
    case 0xE: return 1.0 - tri_occ(-d21, -d11, -d12);
    case 0xD: return 1.0 - tri_occ(-d11, -d12, -d22);
    case 0xB: return 1.0 - tri_occ(-d12, -d22, -d21);
    case 0x7: return 1.0 - tri_occ(-d22, -d21, -d11);
    case 0x3: return trap_occ(d21, d22, d11, d12);
    case 0x6: return trap_occ(d11, d21, d12, d22);
    case 0x9: return trap_occ(d12, d22, d11, d21);
    case 0xC: return trap_occ(d11, d12, d21, d22);
    case 0x5: return tri_occ(d11, d12, d22) + tri_occ(d22, d21, d11);
    case 0xA: return tri_occ(d21, d11, d12) + tri_occ(d12, d22, d21);
    case 0xF: return 1.0;
    }
    return 0.0;
}

/* ------------------------------------------------------------ quantities */

typedef struct {
    double *src, *dst, *phi, *volume, *nx, *ny;
    uint8_t *cell, *body, *mask;
    int w, h;
    double ox, oy, hx;
    int present;
} quantity;

struct ifo_solver {
    int variant, w, h;
    double hx, rho_air, rho_soot, diffusion, t_amb, g;
    quantity q[4];
    double *r, *p, *z, *s, *precon, *adiag, *aplusx, *aplusy, *udens, *vdens;
    ifo_body bodies[256];
    int nbodies;
    int pinned, pinned_heat;
    ifo_pcg_stats st_pressure, st_heat;
    int *stack;
    /* step 8: particles (ParticleQuantities, 8-flip/Fluid.cpp:692-731) */
    double *px, *py, *prop[4], *weight;
    int *counts;
    int np, np_cap, particles_ready;
    uint32_t rng;
    double inflow[16][8];
    int ninflow;
};

#define AT(qq, x, y) ((qq)->src[(x) + (y) * (qq)->w])

/* FluidQuantity ctor: 3-conjugate-gradients/Fluid.cpp:92-98,
 * 4-solid-boundaries/Fluid.cpp:304-318, 7-variable-density/Fluid.cpp:318-338 */
static void q_init(quantity *q, int variant, int w, int h, double ox, double oy, double hx) {
    size_t n = (size_t)w * h;
    q->w = w; q->h = h; q->ox = ox; q->oy = oy; q->hx = hx; q->present = 1;
    q->src = calloc(n, sizeof(double));
    q->dst = calloc(n, sizeof(double));
    q->phi = calloc((size_t)(w + 1) * (h + 1), sizeof(double));
    q->volume = calloc(n, sizeof(double));
    q->nx = calloc(n, sizeof(double));
    q->ny = calloc(n, sizeof(double));
    q->cell = calloc(n, 1);
    q->body = calloc(n, 1);
    q->mask = calloc(n, 1);
    if (variant >= IFO_CURVED)
        for (size_t i = 0; i < n; i++) q->volume[i] = 1.0;
}

static void q_free(quantity *q) {
    if (!q->present) return;
    free(q->src); free(q->dst); free(q->phi); free(q->volume);
    free(q->nx); free(q->ny); free(q->cell); free(q->body); free(q->mask);
}

/* lerp: 3-conjugate-gradients/Fluid.cpp:51-53, 121-133 */
static inline double lerp1(double a, double b, double x) { return a * (1.0 - x) + b * x; }
static double q_lerp(const quantity *q, double x, double y) {
    x = smin(smax(x - q->ox, 0.0), q->w - 1.001);
    y = smin(smax(y - q->oy, 0.0), q->h - 1.001);
    int ix = (int)x, iy = (int)y;
    x -= ix;
    y -= iy;
    double x00 = AT(q, ix + 0, iy + 0), x10 = AT(q, ix + 1, iy + 0);
    double x01 = AT(q, ix + 0, iy + 1), x11 = AT(q, ix + 1, iy + 1);
    return lerp1(lerp1(x00, x10, x), lerp1(x01, x11, x), y);
}

/* cerp: 3-conjugate-gradients/Fluid.cpp:55-69, 135-152 */
static double cerp1(double a, double b, double c, double d, double x) {
    double xsq = x * x;
    double xcu = xsq * x;
    double minV = smin(a, smin(b, smin(c, d)));
    double maxV = smax(a, smax(b, smax(c, d)));
    double t = a * (0.0 - 0.5 * x + 1.0 * xsq - 0.5 * xcu) +
               b * (1.0 + 0.0 * x - 2.5 * xsq + 1.5 * xcu) +
               c * (0.0 + 0.5 * x + 2.0 * xsq - 1.5 * xcu) +
               d * (0.0 + 0.0 * x - 0.5 * xsq + 0.5 * xcu);
    return smin(smax(t, minV), maxV);
}
static double q_cerp(const quantity *q, double x, double y) {
    x = smin(smax(x - q->ox, 0.0), q->w - 1.001);
    y = smin(smax(y - q->oy, 0.0), q->h - 1.001);
    int ix = (int)x, iy = (int)y;
    x -= ix;
    y -= iy;
    int x0 = imax(ix - 1, 0), x1 = ix, x2 = ix + 1, x3 = imin(ix + 2, q->w - 1);
    int y0 = imax(iy - 1, 0), y1 = iy, y2 = iy + 1, y3 = imin(iy + 2, q->h - 1);
    double q0 = cerp1(AT(q, x0, y0), AT(q, x1, y0), AT(q, x2, y0), AT(q, x3, y0), x);
    double q1 = cerp1(AT(q, x0, y1), AT(q, x1, y1), AT(q, x2, y1), AT(q, x3, y1), x);
    double q2 = cerp1(AT(q, x0, y2), AT(q, x1, y2), AT(q, x2, y2), AT(q, x3, y2), x);
    double q3 = cerp1(AT(q, x0, y3), AT(q, x1, y3), AT(q, x2, y3), AT(q, x3, y3), x);
    return cerp1(q0, q1, q2, q3, y);
}

/* rungeKutta3: 3-conjugate-gradients/Fluid.cpp:71-89 (the last stage is not
 * divided by hx, as in the reference) */
static void rk3(const quantity *q, double *px, double *py, double dt,
                const quantity *u, const quantity *v) {
    double x = *px, y = *py;
    double firstU = q_lerp(u, x, y) / q->hx;
    double firstV = q_lerp(v, x, y) / q->hx;
    double midX = x - 0.5 * dt * firstU;
    double midY = y - 0.5 * dt * firstV;
    double midU = q_lerp(u, midX, midY) / q->hx;
    double midV = q_lerp(v, midX, midY) / q->hx;
    double lastX = x - 0.75 * dt * midU;
    double lastY = y - 0.75 * dt * midV;
    double lastU = q_lerp(u, lastX, lastY);
    double lastV = q_lerp(v, lastX, lastY);
    x -= dt * ((2.0 / 9.0) * firstU + (3.0 / 9.0) * midU + (4.0 / 9.0) * lastU);
    y -= dt * ((2.0 / 9.0) * firstV + (3.0 / 9.0) * midV + (4.0 / 9.0) * lastV);
    *px = x;
    *py = y;
}

/* backProject: 4-solid-boundaries/Fluid.cpp:393-404 */
static void back_project(const ifo_solver *s, const quantity *q, double *px, double *py) {
    double x = *px, y = *py;
    int rx = imin(imax((int)(x - q->ox), 0), q->w - 1);
    int ry = imin(imax((int)(y - q->oy), 0), q->h - 1);
    if (q->cell[rx + ry * q->w] != CELL_FLUID) {
        x = (x - q->ox) * q->hx;
        y = (y - q->oy) * q->hx;
        body_closest(&s->bodies[q->body[rx + ry * q->w]], &x, &y);
        x = x / q->hx + q->ox;
        y = y / q->hx + q->oy;
    }
    *px = x;
    *py = y;
}

/* advect: 3-conjugate-gradients/Fluid.cpp:154-165 (all cells),
 * 4-solid-boundaries/Fluid.cpp:406-427 (fluid cells, back projection) */
static void q_advect(const ifo_solver *s, quantity *q, double dt) {
    const quantity *u = &s->q[IFO_QU], *v = &s->q[IFO_QV];
    int solid = s->variant >= IFO_SOLID;
    if (s->variant == IFO_GS_EULER) {  /* euler + lerp: 1-matrixless/Fluid.cpp:65-73, 124-138 */
        for (int iy = 0, idx = 0; iy < q->h; iy++)
            for (int ix = 0; ix < q->w; ix++, idx++) {
                double x = ix + q->ox, y = iy + q->oy;
                double uVel = q_lerp(u, x, y) / q->hx;
                double vVel = q_lerp(v, x, y) / q->hx;
                x -= uVel * dt;
                y -= vVel * dt;
                q->dst[idx] = q_lerp(q, x, y);
            }
        return;
    }
    for (int iy = 0, idx = 0; iy < q->h; iy++) {
        for (int ix = 0; ix < q->w; ix++, idx++) {
            if (solid && q->cell[idx] != CELL_FLUID) continue;
            double x = ix + q->ox;
            double y = iy + q->oy;
            rk3(q, &x, &y, dt, u, v);
            if (solid) back_project(s, q, &x, &y);
            q->dst[idx] = q_cerp(q, x, y);
        }
    }
}

/* addInflow: 3-conjugate-gradients/Fluid.cpp:167-184.  The x loop bound is
 * the grid height as in the reference; cells are addressed by the flat index
 * x + y*w, and a flat index beyond the array is skipped. */
static void q_add_inflow_flat(quantity *q, double x0, double y0, double x1, double y1, double val);
static void q_add_inflow(quantity *q, double x0, double y0, double x1, double y1, double val) {
    int ix0 = (int)(x0 / q->hx - q->ox);
    int iy0 = (int)(y0 / q->hx - q->oy);
    int ix1 = (int)(x1 / q->hx - q->ox);
    int iy1 = (int)(y1 / q->hx - q->oy);
    long n = (long)q->w * q->h;
    for (int y = imax(iy0, 0); y < imin(iy1, q->h); y++) {
        for (int x = imax(ix0, 0); x < imin(ix1, q->h); x++) {
            double l = length2((2.0 * (x + 0.5) * q->hx - (x0 + x1)) / (x1 - x0),
                               (2.0 * (y + 0.5) * q->hx - (y0 + y1)) / (y1 - y0));
            double vi = cubic_pulse(l) * val;
            long flat = (long)x + (long)y * q->w;
            if (flat >= n) continue;
            if (fabs(q->src[flat]) < fabs(vi)) q->src[flat] = vi;
        }
    }
}

/* Step 1's addInflow sets the value itself, without the pulse
 * (1-matrixless/Fluid.cpp:141-151); same bounds and flat-index rule. */
static void q_add_inflow_flat(quantity *q, double x0, double y0, double x1, double y1, double val) {
    int ix0 = (int)(x0 / q->hx - q->ox);
    int iy0 = (int)(y0 / q->hx - q->oy);
    int ix1 = (int)(x1 / q->hx - q->ox);
    int iy1 = (int)(y1 / q->hx - q->oy);
    long n = (long)q->w * q->h;
    for (int y = imax(iy0, 0); y < imin(iy1, q->h); y++)
        for (int x = imax(ix0, 0); x < imin(ix1, q->h); x++) {
            long flat = (long)x + (long)y * q->w;
            if (flat >= n) continue;
            if (fabs(q->src[flat]) < fabs(val)) q->src[flat] = val;
        }
}

/* fillSolidFields: 4-solid-boundaries/Fluid.cpp:449-480 (binary cells),
 * 7-variable-density/Fluid.cpp:475-522 (distance grid, fractional volume) */
static void q_fill_solid(const ifo_solver *s, quantity *q) {
    const ifo_body *B = s->bodies;
    int nb = s->nbodies;
    if (nb == 0) return;
    if (s->variant >= IFO_CURVED) {
        for (int iy = 0, idx = 0; iy <= q->h; iy++) {
            for (int ix = 0; ix <= q->w; ix++, idx++) {
                double x = (ix + q->ox - 0.5) * q->hx;
                double y = (iy + q->oy - 0.5) * q->hx;
                q->phi[idx] = body_distance(&B[0], x, y);
                for (int i = 1; i < nb; i++)
                    q->phi[idx] = smin(q->phi[idx], body_distance(&B[i], x, y));
            }
        }
    }
    for (int iy = 0, idx = 0; iy < q->h; iy++) {
        for (int ix = 0; ix < q->w; ix++, idx++) {
            double x = (ix + q->ox) * q->hx;
            double y = (iy + q->oy) * q->hx;
            q->body[idx] = 0;
            double d = body_distance(&B[0], x, y);
            for (int i = 1; i < nb; i++) {
                double id = body_distance(&B[i], x, y);
                if (id < d) {
                    q->body[idx] = (uint8_t)i;
                    d = id;
                }
            }
            if (s->variant >= IFO_CURVED) {
                int idxp = ix + iy * (q->w + 1);
                q->volume[idx] = 1.0 - occupancy(q->phi[idxp], q->phi[idxp + 1],
                                                 q->phi[idxp + q->w + 1], q->phi[idxp + q->w + 2]);
                if (q->volume[idx] < 0.01) q->volume[idx] = 0.0;
                body_normal(&B[q->body[idx]], &q->nx[idx], &q->ny[idx], x, y);
                q->cell[idx] = (q->volume[idx] == 0.0) ? CELL_SOLID : CELL_FLUID;
            } else {
                q->cell[idx] = (d < 0.0) ? CELL_SOLID : CELL_FLUID;
                body_normal(&B[q->body[idx]], &q->nx[idx], &q->ny[idx], x, y);
            }
        }
    }
}

/* extrapolate / fillSolidMask / extrapolateNormal / freeNeighbour:
 * 4-solid-boundaries/Fluid.cpp:508-587.  LIFO stack as in the reference.
 * Accesses that would leave the array (only possible when a solid touches the
 * outer ring) are skipped. */
static void q_free_neighbour(quantity *q, int idx, int *stack, int *top, int m) {
    q->mask[idx] &= (uint8_t)~m;
    if (q->cell[idx] != CELL_FLUID && q->mask[idx] == 0) stack[(*top)++] = idx;
}
static void q_extrapolate(ifo_solver *s, quantity *q) {
    int w = q->w, h = q->h, n = w * h;
    for (int y = 1; y < h - 1; y++) {
        for (int x = 1; x < w - 1; x++) {
            int idx = x + y * w;
            if (q->cell[idx] == CELL_FLUID) continue;
            double nx = q->nx[idx], ny = q->ny[idx];
            q->mask[idx] = 0;
            if (nx != 0.0 && q->cell[idx + sgn(nx)] != CELL_FLUID) q->mask[idx] |= 1;
            if (ny != 0.0 && q->cell[idx + sgn(ny) * w] != CELL_FLUID) q->mask[idx] |= 2;
        }
    }
    int *stack = s->stack;
    int top = 0;
    for (int y = 1; y < h - 1; y++)
        for (int x = 1; x < w - 1; x++) {
            int idx = x + y * w;
            if (q->cell[idx] != CELL_FLUID && q->mask[idx] == 0) stack[top++] = idx;
        }
    long guard = 0;
    while (top > 0 && guard++ < 16L * n + 16) {
        int idx = stack[--top];
        int ix = idx + sgn(q->nx[idx]), iy = idx + sgn(q->ny[idx]) * w;
        if (ix < 0 || ix >= n || iy < 0 || iy >= n) continue;
        double nx = q->nx[idx], ny = q->ny[idx];
        q->src[idx] = (fabs(nx) * q->src[ix] + fabs(ny) * q->src[iy]) / (fabs(nx) + fabs(ny));
        if (idx - 1 >= 0 && q->nx[idx - 1] > 0.0) q_free_neighbour(q, idx - 1, stack, &top, 1);
        if (idx + 1 < n && q->nx[idx + 1] < 0.0) q_free_neighbour(q, idx + 1, stack, &top, 1);
        if (idx - w >= 0 && q->ny[idx - w] > 0.0) q_free_neighbour(q, idx - w, stack, &top, 2);
        if (idx + w < n && q->ny[idx + w] < 0.0) q_free_neighbour(q, idx + w, stack, &top, 2);
    }
}

/* --------------------------------------------------------------- solver */

ifo_solver *ifo_create(int variant, int w, int h, double density_air,
                       double density_soot, double diffusion) {
    if (variant < IFO_GS_EULER || variant > IFO_FLIP || w < 2 || h < 2) return NULL;
    ifo_solver *s = calloc(1, sizeof(ifo_solver));
    s->variant = variant;
    s->w = w;
    s->h = h;
    s->rho_air = density_air;
    s->rho_soot = density_soot;
    s->diffusion = diffusion;
    s->t_amb = 294.0;  /* 7-variable-density/Fluid.cpp:950-951 */
    s->g = 9.81;
    s->hx = 1.0 / imin(w, h);
    s->pinned = -1;
    s->pinned_heat = -1;
    s->st_pressure.status = IFO_PCG_INITIAL;
    s->st_heat.status = IFO_PCG_INITIAL;
    q_init(&s->q[IFO_QD], variant, w, h, 0.5, 0.5, s->hx);
    if (variant >= IFO_HEAT) q_init(&s->q[IFO_QT], variant, w, h, 0.5, 0.5, s->hx);
    q_init(&s->q[IFO_QU], variant, w + 1, h, 0.0, 0.5, s->hx);
    q_init(&s->q[IFO_QV], variant, w, h + 1, 0.5, 0.0, s->hx);
    if (variant >= IFO_HEAT)
        for (int i = 0; i < w * h; i++) s->q[IFO_QT].src[i] = s->t_amb;
    size_t n = (size_t)w * h;
    s->r = calloc(n, 8); s->p = calloc(n, 8); s->z = calloc(n, 8); s->s = calloc(n, 8);
    s->precon = calloc(n, 8); s->adiag = calloc(n, 8);
    s->aplusx = calloc(n, 8); s->aplusy = calloc(n, 8);
    s->udens = calloc((size_t)(w + 1) * h, 8);
    s->vdens = calloc((size_t)w * (h + 1), 8);
    s->stack = malloc(sizeof(int) * (16 * (size_t)(w + 2) * (h + 2) + 64));
    s->rng = 0xBA5EBA11u;  /* frand's seed, 8-flip/Fluid.cpp:39 */
    if (variant == IFO_FLIP) {
        s->np_cap = w * h * 12;  /* _maxParticles = w*h*_MaxPerCell */
        s->px = calloc((size_t)s->np_cap, 8);
        s->py = calloc((size_t)s->np_cap, 8);
        for (int k = 0; k < 4; k++) s->prop[k] = calloc((size_t)s->np_cap, 8);
        s->weight = calloc((size_t)(w + 1) * (h + 1), 8);
        s->counts = calloc(n, sizeof(int));
    }
    return s;
}

void ifo_destroy(ifo_solver *s) {
    if (!s) return;
    for (int i = 0; i < 4; i++) q_free(&s->q[i]);
    free(s->r); free(s->p); free(s->z); free(s->s); free(s->precon);
    free(s->adiag); free(s->aplusx); free(s->aplusy); free(s->udens); free(s->vdens);
    free(s->stack);
    free(s->px); free(s->py); free(s->weight); free(s->counts);
    for (int k = 0; k < 4; k++) free(s->prop[k]);
    free(s);
}

int ifo_set_bodies(ifo_solver *s, const ifo_body *bodies, int n) {
    if (n < 0 || n > 256) return -1;
    if (n) memcpy(s->bodies, bodies, sizeof(ifo_body) * (size_t)n);
    s->nbodies = n;
    return 0;
}
void ifo_get_bodies(const ifo_solver *s, ifo_body *bodies) {
    memcpy(bodies, s->bodies, sizeof(ifo_body) * (size_t)s->nbodies);
}

/* SolidBody::update: 4-solid-boundaries/Fluid.cpp:140-148 */
void ifo_advance_bodies(ifo_solver *s, double dt) {
    for (int i = 0; i < s->nbodies; i++) {
        ifo_body *b = &s->bodies[i];
        b->pos_x += b->vel_x * dt;
        b->pos_y += b->vel_y * dt;
        b->theta += b->vel_theta * dt;
    }
}

/* FluidSolver::addInflow: 3-conjugate-gradients/Fluid.cpp:449-453,
 * 7-variable-density/Fluid.cpp:1036-1041 */
void ifo_add_inflow(ifo_solver *s, double x, double y, double w, double h,
                    double d, double t, double u, double v) {
    if (s->variant == IFO_FLIP) {  /* applied inside the next update, after copy() */
        if (s->ninflow < 16) {
            double *f = s->inflow[s->ninflow++];
            f[0] = x; f[1] = y; f[2] = w; f[3] = h; f[4] = d; f[5] = t; f[6] = u; f[7] = v;
        }
        return;
    }
    if (s->variant == IFO_GS_EULER) {
        q_add_inflow_flat(&s->q[IFO_QD], x, y, x + w, y + h, d);
        q_add_inflow_flat(&s->q[IFO_QU], x, y, x + w, y + h, u);
        q_add_inflow_flat(&s->q[IFO_QV], x, y, x + w, y + h, v);
        return;
    }
    q_add_inflow(&s->q[IFO_QD], x, y, x + w, y + h, d);
    if (s->variant >= IFO_HEAT) q_add_inflow(&s->q[IFO_QT], x, y, x + w, y + h, t);
    q_add_inflow(&s->q[IFO_QU], x, y, x + w, y + h, u);
    q_add_inflow(&s->q[IFO_QV], x, y, x + w, y + h, v);
}

#define SU(x, y) (U->src[(x) + (y) * U->w])
#define SV(x, y) (V->src[(x) + (y) * V->w])

/* buildRhs: 3-conjugate-gradients/Fluid.cpp:208-217,
 * 4-solid-boundaries/Fluid.cpp:614-627, 7-variable-density/Fluid.cpp:624-653 */
static void build_rhs(ifo_solver *s) {
    const quantity *D = &s->q[IFO_QD], *U = &s->q[IFO_QU], *V = &s->q[IFO_QV];
    double scale = 1.0 / s->hx;
    int w = s->w, h = s->h;
    for (int y = 0, idx = 0; y < h; y++) {
        for (int x = 0; x < w; x++, idx++) {
            if (s->variant <= IFO_PLAIN) {  /* 1-matrixless/Fluid.cpp:176-186 as well */
                s->r[idx] = -scale * (SU(x + 1, y) - SU(x, y) + SV(x, y + 1) - SV(x, y));
            } else if (s->variant == IFO_SOLID) {
                if (D->cell[idx] == CELL_FLUID)
                    s->r[idx] = -scale * (SU(x + 1, y) - SU(x, y) + SV(x, y + 1) - SV(x, y));
                else
                    s->r[idx] = 0.0;
            } else {
                if (D->cell[idx] == CELL_FLUID) {
                    double uv0 = U->volume[x + y * U->w], uv1 = U->volume[x + 1 + y * U->w];
                    double vv0 = V->volume[x + y * V->w], vv1 = V->volume[x + (y + 1) * V->w];
                    s->r[idx] = -scale * (uv1 * SU(x + 1, y) - uv0 * SU(x, y) +
                                          vv1 * SV(x, y + 1) - vv0 * SV(x, y));
                    double vol = D->volume[idx];
                    if (s->nbodies == 0) continue;
                    const uint8_t *body = D->body;
                    if (x > 0)
                        s->r[idx] -= (uv0 - vol) * body_vel_x(&s->bodies[body[idx - 1]], x * s->hx, (y + 0.5) * s->hx);
                    if (y > 0)
                        s->r[idx] -= (vv0 - vol) * body_vel_y(&s->bodies[body[idx - w]], (x + 0.5) * s->hx, y * s->hx);
                    if (x < w - 1)
                        s->r[idx] += (uv1 - vol) * body_vel_x(&s->bodies[body[idx + 1]], (x + 1.0) * s->hx, (y + 0.5) * s->hx);
                    if (y < h - 1)
                        s->r[idx] += (vv1 - vol) * body_vel_y(&s->bodies[body[idx + w]], (x + 0.5) * s->hx, (y + 1.0) * s->hx);
                } else
                    s->r[idx] = 0.0;
            }
        }
    }
}

/* computeDensities: 7-variable-density/Fluid.cpp:658-675 */
static void compute_densities(ifo_solver *s) {
    const quantity *D = &s->q[IFO_QD], *T = &s->q[IFO_QT];
    int w = s->w, h = s->h;
    double alpha = (s->rho_soot - s->rho_air) / s->rho_air;
    memset(s->udens, 0, sizeof(double) * (size_t)(w + 1) * h);
    memset(s->vdens, 0, sizeof(double) * (size_t)w * (h + 1));
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            double density = s->rho_air * s->t_amb / T->src[x + y * w] * (1.0 + alpha * D->src[x + y * w]);
            density = smax(density, 0.05 * s->rho_air);
            s->udens[x + y * (w + 1)] += 0.5 * density;
            s->vdens[x + y * w] += 0.5 * density;
            s->udens[x + 1 + y * (w + 1)] += 0.5 * density;
            s->vdens[x + (y + 1) * w] += 0.5 * density;
        }
}

/* buildPressureMatrix: 3-conjugate-gradients/Fluid.cpp:222-244,
 * 4-solid-boundaries/Fluid.cpp:629-654, 5-curved-boundaries/Fluid.cpp:686-713,
 * 6-heat/Fluid.cpp:649-676, 7-variable-density/Fluid.cpp:680-707.  Step 7
 * reads the v-face density at the u-grid index x + (y+1)*(w+1); a read beyond
 * the v-density array is skipped (treated as a missing face). */
static void build_matrix(ifo_solver *s, double dt) {
    const quantity *D = &s->q[IFO_QD], *U = &s->q[IFO_QU], *V = &s->q[IFO_QV];
    int w = s->w, h = s->h;
    size_t n = (size_t)w * h;
    if (s->variant == IFO_PLAIN) {
        double scale = dt / (s->rho_air * s->hx * s->hx);
        memset(s->adiag, 0, n * 8);
        for (int y = 0, idx = 0; y < h; y++)
            for (int x = 0; x < w; x++, idx++) {
                if (x < w - 1) {
                    s->adiag[idx] += scale;
                    s->adiag[idx + 1] += scale;
                    s->aplusx[idx] = -scale;
                } else
                    s->aplusx[idx] = 0.0;
                if (y < h - 1) {
                    s->adiag[idx] += scale;
                    s->adiag[idx + w] += scale;
                    s->aplusy[idx] = -scale;
                } else
                    s->aplusy[idx] = 0.0;
            }
        return;
    }
    double scale = (s->variant >= IFO_VARDENS) ? dt / (s->hx * s->hx)
                                               : dt / (s->rho_air * s->hx * s->hx);
    memset(s->adiag, 0, n * 8);
    memset(s->aplusx, 0, n * 8);
    memset(s->aplusy, 0, n * 8);
    const uint8_t *cell = D->cell;
    long vdn = (long)w * (h + 1);
    for (int y = 0, idx = 0; y < h; y++)
        for (int x = 0; x < w; x++, idx++) {
            if (cell[idx] != CELL_FLUID) continue;
            if (x < w - 1 && cell[idx + 1] == CELL_FLUID) {
                double f;
                if (s->variant == IFO_SOLID) f = scale;
                else if (s->variant >= IFO_VARDENS)
                    f = scale * U->volume[x + 1 + y * U->w] / s->udens[x + 1 + y * (w + 1)];
                else f = scale * U->volume[x + 1 + y * U->w];
                s->adiag[idx] += f;
                s->adiag[idx + 1] += f;
                s->aplusx[idx] = -f;
            }
            if (y < h - 1 && cell[idx + w] == CELL_FLUID) {
                double f;
                if (s->variant == IFO_SOLID) f = scale;
                else if (s->variant >= IFO_VARDENS) {
                    long vi = (long)x + (long)(y + 1) * (w + 1);
                    if (vi >= vdn) continue;
                    f = scale * V->volume[x + (y + 1) * V->w] / s->vdens[vi];
                } else f = scale * V->volume[x + (y + 1) * V->w];
                s->adiag[idx] += f;
                s->adiag[idx + w] += f;
                s->aplusy[idx] = -f;
            }
        }
}

/* buildHeatDiffusionMatrix: 7-variable-density/Fluid.cpp:709-737 */
static void build_heat_matrix(ifo_solver *s, double dt) {
    int w = s->w, h = s->h;
    size_t n = (size_t)w * h;
    for (size_t i = 0; i < n; i++) s->adiag[i] = 1.0;
    memset(s->aplusx, 0, n * 8);
    memset(s->aplusy, 0, n * 8);
    const uint8_t *cell = s->q[IFO_QD].cell;
    double scale = s->diffusion * dt * 1.0 / (s->hx * s->hx);
    for (int y = 0, idx = 0; y < h; y++)
        for (int x = 0; x < w; x++, idx++) {
            if (cell[idx] != CELL_FLUID) continue;
            if (x < w - 1 && cell[idx + 1] == CELL_FLUID) {
                s->adiag[idx] += scale;
                s->adiag[idx + 1] += scale;
                s->aplusx[idx] = -scale;
            }
            if (y < h - 1 && cell[idx + w] == CELL_FLUID) {
                s->adiag[idx] += scale;
                s->adiag[idx + w] += scale;
                s->aplusy[idx] = -scale;
            }
        }
}

/* buildPreconditioner (MIC(0)): 3-conjugate-gradients/Fluid.cpp:247-272,
 * masked in 4-solid-boundaries/Fluid.cpp:656-685 */
static void build_precon(ifo_solver *s) {
    int w = s->w, h = s->h;
    int masked = s->variant >= IFO_SOLID;
    const uint8_t *cell = s->q[IFO_QD].cell;
    for (int y = 0, idx = 0; y < h; y++)
        for (int x = 0; x < w; x++, idx++) {
            if (masked && cell[idx] != CELL_FLUID) continue;
            double e = s->adiag[idx];
            if (x > 0 && (!masked || cell[idx - 1] == CELL_FLUID)) {
                double px = s->aplusx[idx - 1] * s->precon[idx - 1];
                double py = s->aplusy[idx - 1] * s->precon[idx - 1];
                e = e - (px * px + MIC_TAU * px * py);
            }
            if (y > 0 && (!masked || cell[idx - w] == CELL_FLUID)) {
                double px = s->aplusx[idx - w] * s->precon[idx - w];
                double py = s->aplusy[idx - w] * s->precon[idx - w];
                e = e - (py * py + MIC_TAU * px * py);
            }
            if (e < MIC_SIGMA * s->adiag[idx]) e = s->adiag[idx];
            s->precon[idx] = 1.0 / sqrt(e);
        }
}

/* applyPreconditioner: 3-conjugate-gradients/Fluid.cpp:275-304,
 * masked in 4-solid-boundaries/Fluid.cpp:687-721 */
static void apply_precon(ifo_solver *s, double *dst, const double *a) {
    int w = s->w, h = s->h;
    int masked = s->variant >= IFO_SOLID;
    const uint8_t *cell = s->q[IFO_QD].cell;
    const double *ax = s->aplusx, *ay = s->aplusy, *pc = s->precon;
    for (int y = 0, idx = 0; y < h; y++)
        for (int x = 0; x < w; x++, idx++) {
            if (masked && cell[idx] != CELL_FLUID) continue;
            double t = a[idx];
            if (x > 0 && (!masked || cell[idx - 1] == CELL_FLUID))
                t -= ax[idx - 1] * pc[idx - 1] * dst[idx - 1];
            if (y > 0 && (!masked || cell[idx - w] == CELL_FLUID))
                t -= ay[idx - w] * pc[idx - w] * dst[idx - w];
            dst[idx] = t * pc[idx];
        }
    for (int y = h - 1; y >= 0; y--)
        for (int x = w - 1; x >= 0; x--) {
            int idx = x + y * w;
            if (masked && cell[idx] != CELL_FLUID) continue;
            double t = dst[idx];
            if (x < w - 1 && (!masked || cell[idx + 1] == CELL_FLUID))
                t -= ax[idx] * pc[idx] * dst[idx + 1];
            if (y < h - 1 && (!masked || cell[idx + w] == CELL_FLUID))
                t -= ay[idx] * pc[idx] * dst[idx + w];
            dst[idx] = t * pc[idx];
        }
}

/* dotProduct / scaledAdd / infinityNorm: 3-conjugate-gradients/Fluid.cpp:307-346;
 * masked to fluid cells from 6-heat/Fluid.cpp:781-826 on */
static double dot(const ifo_solver *s, const double *a, const double *b) {
    int n = s->w * s->h;
    const uint8_t *cell = s->q[IFO_QD].cell;
    int masked = s->variant >= IFO_HEAT;
    double r = 0.0;
    for (int i = 0; i < n; i++)
        if (!masked || cell[i] == CELL_FLUID) r += a[i] * b[i];
    return r;
}
static void scaled_add(const ifo_solver *s, double *dst, const double *a, const double *b, double k) {
    int n = s->w * s->h;
    const uint8_t *cell = s->q[IFO_QD].cell;
    int masked = s->variant >= IFO_HEAT;
    for (int i = 0; i < n; i++)
        if (!masked || cell[i] == CELL_FLUID) dst[i] = a[i] + b[i] * k;
}
static double inf_norm(const ifo_solver *s, const double *a) {
    int n = s->w * s->h;
    const uint8_t *cell = s->q[IFO_QD].cell;
    int masked = s->variant >= IFO_HEAT;
    double m = 0.0;
    for (int i = 0; i < n; i++)
        if (!masked || cell[i] == CELL_FLUID) m = smax(m, fabs(a[i]));
    return m;
}

/* matrixVectorProduct: 3-conjugate-gradients/Fluid.cpp:315-332 (never masked) */
static void matvec(const ifo_solver *s, double *dst, const double *b) {
    int w = s->w, h = s->h;
    for (int y = 0, idx = 0; y < h; y++)
        for (int x = 0; x < w; x++, idx++) {
            double t = s->adiag[idx] * b[idx];
            if (x > 0) t += s->aplusx[idx - 1] * b[idx - 1];
            if (y > 0) t += s->aplusy[idx - w] * b[idx - w];
            if (x < w - 1) t += s->aplusx[idx] * b[idx + 1];
            if (y < h - 1) t += s->aplusy[idx] * b[idx + w];
            dst[idx] = t;
        }
}

/* project (PCG): 3-conjugate-gradients/Fluid.cpp:349-380 */
static void project(ifo_solver *s, int limit, int pinned, ifo_pcg_stats *st) {
    size_t n = (size_t)s->w * s->h;
    memset(s->p, 0, n * 8);
    apply_precon(s, s->z, s->r);
    memcpy(s->s, s->z, n * 8);
    double maxError = inf_norm(s, s->r);
    st->max_error = maxError;
    st->iterations = 0;
    if (pinned >= 0 ? pinned == 0 : maxError < PCG_TOL) {
        st->status = IFO_PCG_INITIAL;
        return;
    }
    double sigma = dot(s, s->z, s->r);
    for (int iter = 0; iter < limit; iter++) {
        matvec(s, s->z, s->s);
        double alpha = sigma / dot(s, s->z, s->s);
        scaled_add(s, s->p, s->p, s->s, alpha);
        scaled_add(s, s->r, s->r, s->z, -alpha);
        maxError = inf_norm(s, s->r);
        st->max_error = maxError;
        st->iterations = iter + 1;
        if (pinned >= 0 ? iter + 1 >= pinned : maxError < PCG_TOL) {
            st->status = IFO_PCG_CONVERGED;
            return;
        }
        apply_precon(s, s->z, s->r);
        double sigmaNew = dot(s, s->z, s->r);
        scaled_add(s, s->s, s->z, s->s, sigmaNew / sigma);
        sigma = sigmaNew;
    }
    st->status = IFO_PCG_CAP;
}

/* applyPressure: 3-conjugate-gradients/Fluid.cpp:382-398,
 * 4-solid-boundaries/Fluid.cpp:794-809, 7-variable-density/Fluid.cpp:891-906 */
static void apply_pressure(ifo_solver *s, double dt) {
    quantity *U = &s->q[IFO_QU], *V = &s->q[IFO_QV];
    const uint8_t *cell = s->q[IFO_QD].cell;
    int w = s->w, h = s->h;
    int masked = s->variant >= IFO_SOLID;
    if (s->variant >= IFO_VARDENS) {
        double scale = dt / s->hx;
        for (int y = 0, idx = 0; y < h; y++)
            for (int x = 0; x < w; x++, idx++) {
                if (cell[idx] != CELL_FLUID) continue;
                SU(x, y) -= scale * s->p[idx] / s->udens[x + y * (w + 1)];
                SV(x, y) -= scale * s->p[idx] / s->vdens[x + y * w];
                SU(x + 1, y) += scale * s->p[idx] / s->udens[x + 1 + y * (w + 1)];
                SV(x, y + 1) += scale * s->p[idx] / s->vdens[x + (y + 1) * w];
            }
        return;
    }
    double scale = dt / (s->rho_air * s->hx);
    for (int y = 0, idx = 0; y < h; y++)
        for (int x = 0; x < w; x++, idx++) {
            if (masked && cell[idx] != CELL_FLUID) continue;
            SU(x, y) -= scale * s->p[idx];
            SU(x + 1, y) += scale * s->p[idx];
            SV(x, y) -= scale * s->p[idx];
            SV(x, y + 1) += scale * s->p[idx];
        }
    if (!masked) {
        for (int y = 0; y < h; y++) SU(0, y) = SU(w, y) = 0.0;
        for (int x = 0; x < w; x++) SV(x, 0) = SV(x, h) = 0.0;
    }
}

/* setBoundaryCondition: 4-solid-boundaries/Fluid.cpp:812-833 */
static void set_bc(ifo_solver *s) {
    quantity *U = &s->q[IFO_QU], *V = &s->q[IFO_QV];
    const quantity *D = &s->q[IFO_QD];
    int w = s->w, h = s->h;
    double hx = s->hx;
    for (int y = 0, idx = 0; y < h; y++)
        for (int x = 0; x < w; x++, idx++) {
            if (D->cell[idx] == CELL_SOLID) {
                const ifo_body *b = &s->bodies[D->body[idx]];
                SU(x, y) = body_vel_x(b, x * hx, (y + 0.5) * hx);
                SV(x, y) = body_vel_y(b, (x + 0.5) * hx, y * hx);
                SU(x + 1, y) = body_vel_x(b, (x + 1.0) * hx, (y + 0.5) * hx);
                SV(x, y + 1) = body_vel_y(b, (x + 0.5) * hx, (y + 1.0) * hx);
            }
        }
    for (int y = 0; y < h; y++) SU(0, y) = SU(w, y) = 0.0;
    for (int x = 0; x < w; x++) SV(x, 0) = SV(x, h) = 0.0;
}

/* addBuoyancy: 7-variable-density/Fluid.cpp:908-919 */
static void add_buoyancy(ifo_solver *s, double dt) {
    const quantity *D = &s->q[IFO_QD], *T = &s->q[IFO_QT];
    quantity *V = &s->q[IFO_QV];
    int w = s->w, h = s->h;
    double alpha = (s->rho_soot - s->rho_air) / s->rho_air;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            double b = dt * s->g * (alpha * D->src[x + y * w] - (T->src[x + y * w] - s->t_amb) / s->t_amb);
            SV(x, y) += b * 0.5;
            SV(x, y + 1) += b * 0.5;
        }
}

/* heat solve: 7-variable-density/Fluid.cpp:1001-1005 */
static void heat_solve(ifo_solver *s, double dt) {
    size_t n = (size_t)s->w * s->h;
    memcpy(s->r, s->q[IFO_QT].src, n * 8);
    build_heat_matrix(s, dt);
    build_precon(s);
    project(s, 2000, s->pinned_heat, &s->st_heat);
    memcpy(s->q[IFO_QT].src, s->p, n * 8);
}

static void flip(quantity *q) {
    double *t = q->src;
    q->src = q->dst;
    q->dst = t;
}

/* ------------------------------------------------------------ step 8: FLIP
 * ParticleQuantities and the FLIP additions to FluidQuantity
 * (8-flip/Fluid.cpp:37-47, 296-303, 374-389, 472-690, 692-940, 1350-1413). */

#define FLIP_MAX_PER_CELL 12
#define FLIP_MIN_PER_CELL 3
#define FLIP_AVG_PER_CELL 4
#define FLIP_ALPHA 0.001

/* frand: a 31-bit LCG whose new state's top 23 bits are the fraction of a
 * float in [0, 1) (8-flip/Fluid.cpp:38-46; the reference forms the float by
 * bit pattern, which is the same number). */
float ifo_frand(uint32_t *state) {
    *state = (*state * 1103515245u + 12345u) & 0x7FFFFFFFu;
    return (float)(*state >> 8) * 0x1p-23f;
}

/* pointInBody: 8-flip/Fluid.cpp:724-731 (x, y in grid units) */
static int point_in_body(const ifo_solver *s, double x, double y) {
    for (int i = 0; i < s->nbodies; i++)
        if (body_distance(&s->bodies[i], x * s->hx, y * s->hx) < 0.0) return 1;
    return 0;
}

/* gridToParticles: 8-flip/Fluid.cpp:886-897 */
static void grid_to_particles(ifo_solver *s, double alpha) {
    for (int t = 0; t < 4; t++) {
        const quantity *q = &s->q[t];
        double *pr = s->prop[t];
        for (int i = 0; i < s->np; i++) {
            pr[i] *= 1.0 - alpha;
            pr[i] += q_lerp(q, s->px[i], s->py[i]);
        }
    }
}

/* initParticles (8-flip/Fluid.cpp:733-750) followed by the solver ctor's
 * gridToParticles(1.0) (8-flip/Fluid.cpp:1307-1314).  A position is int +
 * float in float arithmetic, as `x + frand()` is in the reference. */
static void flip_init(ifo_solver *s) {
    if (s->particles_ready) return;
    int n = 0;
    for (int y = 0; y < s->h; y++)
        for (int x = 0; x < s->w; x++)
            for (int i = 0; i < FLIP_AVG_PER_CELL; i++) {
                s->px[n] = (double)((float)x + ifo_frand(&s->rng));
                s->py[n] = (double)((float)y + ifo_frand(&s->rng));
                if (!point_in_body(s, s->px[n], s->py[n])) n++;
            }
    s->np = n;
    s->particles_ready = 1;
    grid_to_particles(s, 1.0);
}

/* fromParticles + addSample: hat-filter transfer onto the quantity's grid;
 * nodes without weight turn fluid cells into CELL_EMPTY
 * (8-flip/Fluid.cpp:296-303, 663-690). */
static void sample_add(quantity *q, double *wgt, double value, double x, double y, int ix, int iy) {
    if (ix < 0 || iy < 0 || ix >= q->w || iy >= q->h) return;
    double k = (1.0 - fabs(ix - x)) * (1.0 - fabs(iy - y));
    wgt[ix + iy * q->w] += k;
    q->src[ix + iy * q->w] += k * value;
}
static void from_particles(ifo_solver *s, quantity *q, const double *value) {
    size_t n = (size_t)q->w * q->h;
    double *wgt = s->weight;
    memset(q->src, 0, n * 8);
    memset(wgt, 0, n * 8);
    for (int i = 0; i < s->np; i++) {
        double x = smax(0.5, smin(q->w - 1.5, s->px[i] - q->ox));
        double y = smax(0.5, smin(q->h - 1.5, s->py[i] - q->oy));
        int ix = (int)x, iy = (int)y;
        sample_add(q, wgt, value[i], x, y, ix, iy);
        sample_add(q, wgt, value[i], x, y, ix + 1, iy);
        sample_add(q, wgt, value[i], x, y, ix, iy + 1);
        sample_add(q, wgt, value[i], x, y, ix + 1, iy + 1);
    }
    for (size_t i = 0; i < n; i++) {
        if (wgt[i] != 0.0) q->src[i] /= wgt[i];
        else if (q->cell[i] == CELL_FLUID) q->cell[i] = CELL_EMPTY;
    }
}

/* extrapolate with empty cells: fillSolidMask, extrapolateNormal,
 * extrapolateAverage, freeSolidNeighbour, freeEmptyNeighbour,
 * extrapolateEmptyBorders (8-flip/Fluid.cpp:478-653).  The outer ring is
 * never pushed (mask 0xFF); empty cells take the mean of the neighbours that
 * are fluid when they are popped, so the LIFO order matters here. */
static void flip_free_solid(quantity *q, int idx, int *stack, int *top, int m) {
    if (q->cell[idx] != CELL_SOLID) return;
    q->mask[idx] &= (uint8_t)~m;
    if (q->mask[idx] == 0) stack[(*top)++] = idx;
}
static void flip_free_empty(quantity *q, int idx, int *stack, int *top) {
    if (q->cell[idx] == CELL_EMPTY && q->mask[idx] == 1) {
        q->mask[idx] = 0;
        stack[(*top)++] = idx;
    }
}
static void flip_extrapolate(ifo_solver *s, quantity *q) {
    const int w = q->w, h = q->h;
    uint8_t *c = q->cell, *m = q->mask;
    double *src = q->src;
    for (int x = 0; x < w; x++) m[x] = m[x + (h - 1) * w] = 0xFF;
    for (int y = 0; y < h; y++) m[y * w] = m[y * w + w - 1] = 0xFF;
    for (int y = 1; y < h - 1; y++)
        for (int x = 1; x < w - 1; x++) {
            int idx = x + y * w;
            m[idx] = 0;
            if (c[idx] == CELL_SOLID) {
                double nx = q->nx[idx], ny = q->ny[idx];
                if (nx != 0.0 && c[idx + sgn(nx)] != CELL_FLUID) m[idx] |= 1;
                if (ny != 0.0 && c[idx + sgn(ny) * w] != CELL_FLUID) m[idx] |= 2;
            } else if (c[idx] == CELL_EMPTY) {
                m[idx] = c[idx - 1] != CELL_FLUID && c[idx + 1] != CELL_FLUID &&
                         c[idx - w] != CELL_FLUID && c[idx + w] != CELL_FLUID;
            }
        }
    int *stack = s->stack, top = 0;
    for (int y = 1; y < h - 1; y++)
        for (int x = 1; x < w - 1; x++) {
            int idx = x + y * w;
            if (c[idx] != CELL_FLUID && m[idx] == 0) stack[top++] = idx;
        }
    while (top > 0) {
        int idx = stack[--top];
        if (c[idx] == CELL_EMPTY) {
            double sum = 0.0;
            int k = 0;
            const int nb[4] = {idx - 1, idx + 1, idx - w, idx + w};
            for (int j = 0; j < 4; j++)
                if (c[nb[j]] == CELL_FLUID) {
                    sum += src[nb[j]];
                    k++;
                }
            src[idx] = sum / k;
            c[idx] = CELL_FLUID;
        } else {
            double nx = q->nx[idx], ny = q->ny[idx];
            src[idx] = (fabs(nx) * src[idx + sgn(nx)] + fabs(ny) * src[idx + sgn(ny) * w]) /
                       (fabs(nx) + fabs(ny));
        }
        if (q->nx[idx - 1] > 0.0) flip_free_solid(q, idx - 1, stack, &top, 1);
        if (q->nx[idx + 1] < 0.0) flip_free_solid(q, idx + 1, stack, &top, 1);
        if (q->ny[idx - w] > 0.0) flip_free_solid(q, idx - w, stack, &top, 2);
        if (q->ny[idx + w] < 0.0) flip_free_solid(q, idx + w, stack, &top, 2);
        flip_free_empty(q, idx - 1, stack, &top);
        flip_free_empty(q, idx + 1, stack, &top);
        flip_free_empty(q, idx - w, stack, &top);
        flip_free_empty(q, idx + w, stack, &top);
    }
    /* outer ring: copy the inward neighbour, corners average two ring cells */
    for (int x = 1; x < w - 1; x++) {
        int t = x, b = x + (h - 1) * w;
        if (c[t] == CELL_EMPTY) src[t] = src[t + w];
        if (c[b] == CELL_EMPTY) src[b] = src[b - w];
    }
    for (int y = 1; y < h - 1; y++) {
        int l = y * w, r = y * w + w - 1;
        if (c[l] == CELL_EMPTY) src[l] = src[l + 1];
        if (c[r] == CELL_EMPTY) src[r] = src[r - 1];
    }
    const int tl = 0, tr = w - 1, bl = (h - 1) * w, br = h * w - 1;
    if (c[tl] == CELL_EMPTY) src[tl] = 0.5 * (src[tl + 1] + src[tl + w]);
    if (c[tr] == CELL_EMPTY) src[tr] = 0.5 * (src[tr - 1] + src[tr + w]);
    if (c[bl] == CELL_EMPTY) src[bl] = 0.5 * (src[bl + 1] + src[bl - w]);
    if (c[br] == CELL_EMPTY) src[br] = 0.5 * (src[br - 1] + src[br - w]);
    for (int i = 0; i < w * h; i++)
        if (c[i] == CELL_EMPTY) c[i] = CELL_FLUID;
}

/* countParticles / pruneParticles / seedParticles (8-flip/Fluid.cpp:752-818).
 * Seeding rejects an attempt when particle number `cell index` (not the new
 * particle) lies inside a body, as the reference does. */
static void copy_particle(ifo_solver *s, int dst, int src) {
    s->px[dst] = s->px[src];
    s->py[dst] = s->py[src];
    for (int t = 0; t < 4; t++) s->prop[t][dst] = s->prop[t][src];
}
static void count_prune_seed(ifo_solver *s) {
    const int w = s->w, h = s->h;
    int *cnt = s->counts;
    memset(cnt, 0, sizeof(int) * (size_t)w * h);
    for (int i = 0; i < s->np; i++) {
        int ix = (int)s->px[i], iy = (int)s->py[i];
        if (ix >= 0 && iy >= 0 && ix < w && iy < h) cnt[ix + iy * w]++;
    }
    for (int i = 0; i < s->np; i++) {
        int ix = (int)s->px[i], iy = (int)s->py[i];
        if (ix < 0 || iy < 0 || ix >= w || iy >= h) continue;
        int idx = ix + iy * w;
        if (cnt[idx] > FLIP_MAX_PER_CELL) {
            copy_particle(s, i, --s->np);
            cnt[idx]--;
            i--;
        }
    }
    for (int y = 0, idx = 0; y < h; y++)
        for (int x = 0; x < w; x++, idx++)
            for (int i = 0; i < FLIP_MIN_PER_CELL - cnt[idx]; i++) {
                if (s->np == s->np_cap) return;
                int j = s->np;
                s->px[j] = (double)((float)x + ifo_frand(&s->rng));
                s->py[j] = (double)((float)y + ifo_frand(&s->rng));
                if (point_in_body(s, s->px[idx], s->py[idx])) continue;
                for (int t = 0; t < 4; t++) s->prop[t][j] = q_lerp(&s->q[t], s->px[j], s->py[j]);
                s->np++;
            }
}

/* particlesToGrid: 8-flip/Fluid.cpp:899-912 */
static void particles_to_grid(ifo_solver *s) {
    flip_init(s);
    for (int t = 0; t < 4; t++) {
        from_particles(s, &s->q[t], s->prop[t]);
        flip_extrapolate(s, &s->q[t]);
    }
    count_prune_seed(s);
}

/* copy() of every quantity, then the inflows of this update
 * (8-flip/Fluid.cpp:374-376, 1359-1368) */
static void flip_copy(ifo_solver *s) {
    for (int t = 0; t < 4; t++) {
        quantity *q = &s->q[t];
        memcpy(q->dst, q->src, (size_t)q->w * q->h * 8);
    }
    for (int k = 0; k < s->ninflow; k++) {
        const double *f = s->inflow[k];
        for (int t = 0; t < 4; t++)
            q_add_inflow(&s->q[t], f[0], f[1], f[0] + f[2], f[1] + f[3], f[4 + t]);
    }
    s->ninflow = 0;
}

/* diff(alpha), gridToParticles(alpha), undiff(alpha)
 * (8-flip/Fluid.cpp:378-389, 1394-1409); `dst` holds _old in step 8. */
static void flip_g2p(ifo_solver *s) {
    const double keep = 1.0 - FLIP_ALPHA;
    for (int t = 0; t < 4; t++) {
        quantity *q = &s->q[t];
        for (int i = 0; i < q->w * q->h; i++) q->src[i] -= keep * q->dst[i];
    }
    grid_to_particles(s, FLIP_ALPHA);
    for (int t = 0; t < 4; t++) {
        quantity *q = &s->q[t];
        for (int i = 0; i < q->w * q->h; i++) q->src[i] += keep * q->dst[i];
    }
}

/* ParticleQuantities::advect with the forward rungeKutta3 and backProject
 * (8-flip/Fluid.cpp:820-870, 916-924); the last RK stage is not divided by
 * hx, as in the reference. */
static void particle_advect(ifo_solver *s, double dt) {
    const quantity *u = &s->q[IFO_QU], *v = &s->q[IFO_QV];
    const double hx = s->hx;
    for (int i = 0; i < s->np; i++) {
        double x = s->px[i], y = s->py[i];
        double firstU = q_lerp(u, x, y) / hx;
        double firstV = q_lerp(v, x, y) / hx;
        double midX = x + 0.5 * dt * firstU;
        double midY = y + 0.5 * dt * firstV;
        double midU = q_lerp(u, midX, midY) / hx;
        double midV = q_lerp(v, midX, midY) / hx;
        double lastX = x + 0.75 * dt * midU;
        double lastY = y + 0.75 * dt * midV;
        double lastU = q_lerp(u, lastX, lastY);
        double lastV = q_lerp(v, lastX, lastY);
        x += dt * ((2.0 / 9.0) * firstU + (3.0 / 9.0) * midU + (4.0 / 9.0) * lastU);
        y += dt * ((2.0 / 9.0) * firstV + (3.0 / 9.0) * midV + (4.0 / 9.0) * lastV);
        double d = 1e30;
        int nearest = -1;
        for (int b = 0; b < s->nbodies; b++) {
            double db = body_distance(&s->bodies[b], x * hx, y * hx);
            if (db < d) {
                d = db;
                nearest = b;
            }
        }
        if (d < -1.0) {
            x *= hx;
            y *= hx;
            body_closest(&s->bodies[nearest], &x, &y);
            double nx, ny;
            body_normal(&s->bodies[nearest], &nx, &ny, x, y);
            x -= nx * hx;
            y -= ny * hx;
            x /= hx;
            y /= hx;
        }
        s->px[i] = smax(smin(x, s->w - 0.001), 0.0);
        s->py[i] = smax(smin(y, s->h - 0.001), 0.0);
    }
}

double *ifo_particles(ifo_solver *s, int which, int *count) {
    *count = s->np;
    if (s->variant != IFO_FLIP) return NULL;
    switch (which) {
    case IFO_P_X: return s->px;
    case IFO_P_Y: return s->py;
    case IFO_P_D: case IFO_P_T: case IFO_P_U: case IFO_P_V: return s->prop[which - IFO_P_D];
    default: return NULL;
    }
}
void ifo_set_particle_count(ifo_solver *s, int n) {
    if (s->variant == IFO_FLIP && n >= 0 && n <= s->np_cap) {
        s->np = n;
        s->particles_ready = 1;
    }
}
void ifo_flip_init(ifo_solver *s) {
    if (s->variant == IFO_FLIP) flip_init(s);
}
uint32_t ifo_rng_state(const ifo_solver *s) { return s->rng; }
void ifo_set_rng_state(ifo_solver *s, uint32_t state) { s->rng = state; }

/* project() of steps 1-2: lexicographic Gauss-Seidel on the implicit
 * five-point stencil, walls solid, p kept from the previous step (zeroed only
 * by the constructor), stop when the largest change of a sweep is below 1e-5
 * (1-matrixless/Fluid.cpp:192-240). */
static void gs_project(ifo_solver *s, int limit, double dt) {
    const int w = s->w, h = s->h;
    const double scale = dt / (s->rho_air * s->hx * s->hx);
    double *p = s->p;
    const double *r = s->r;
    double maxDelta = 0.0;
    int sweeps = 0;
    for (int it = 0; it < limit; it++) {
        maxDelta = 0.0;
        for (int y = 0; y < h; y++)
            for (int x = 0; x < w; x++) {
                int idx = x + y * w;
                double diag = 0.0, off = 0.0;
                if (x > 0) { diag += scale; off -= scale * p[idx - 1]; }
                if (y > 0) { diag += scale; off -= scale * p[idx - w]; }
                if (x < w - 1) { diag += scale; off -= scale * p[idx + 1]; }
                if (y < h - 1) { diag += scale; off -= scale * p[idx + w]; }
                double np_ = (r[idx] - off) / diag;
                maxDelta = smax(maxDelta, fabs(p[idx] - np_));
                p[idx] = np_;
            }
        sweeps = it + 1;
        if (maxDelta < 1e-5) {
            s->st_pressure.iterations = sweeps;
            s->st_pressure.status = IFO_PCG_CONVERGED;
            s->st_pressure.max_error = maxDelta;
            return;
        }
    }
    s->st_pressure.iterations = limit;
    s->st_pressure.status = IFO_PCG_CAP;
    s->st_pressure.max_error = maxDelta;
    (void)sweeps;
}

void ifo_phase(ifo_solver *s, int phase, double dt) {
    int v = s->variant;
    switch (phase) {
    case IFO_PH_FILL_SOLID:
        if (v < IFO_SOLID) break;
        q_fill_solid(s, &s->q[IFO_QD]);
        if (v >= IFO_HEAT) q_fill_solid(s, &s->q[IFO_QT]);
        q_fill_solid(s, &s->q[IFO_QU]);
        q_fill_solid(s, &s->q[IFO_QV]);
        break;
    case IFO_PH_HEAT: if (v >= IFO_HEAT) heat_solve(s, dt); break;
    case IFO_PH_EXTRAP_T:
        if (v == IFO_FLIP) flip_extrapolate(s, &s->q[IFO_QT]);
        else if (v >= IFO_HEAT) q_extrapolate(s, &s->q[IFO_QT]);
        break;
    case IFO_PH_BUOYANCY: if (v >= IFO_HEAT) add_buoyancy(s, dt); break;
    case IFO_PH_BC: if (v >= IFO_SOLID) set_bc(s); break;
    case IFO_PH_RHS: build_rhs(s); break;
    case IFO_PH_DENSITIES: if (v >= IFO_VARDENS) compute_densities(s); break;
    case IFO_PH_MATRIX: if (v > IFO_GS) build_matrix(s, dt); break;
    case IFO_PH_PRECON: if (v > IFO_GS) build_precon(s); break;
    case IFO_PH_PROJECT:
        if (v <= IFO_GS) gs_project(s, 600, dt);
        else project(s, v == IFO_PLAIN ? 600 : 2000, s->pinned, &s->st_pressure);
        break;
    case IFO_PH_APPLY_P: apply_pressure(s, dt); break;
    case IFO_PH_EXTRAP_DUV:
        if (v < IFO_SOLID) break;
        if (v == IFO_FLIP) {
            flip_extrapolate(s, &s->q[IFO_QD]);
            flip_extrapolate(s, &s->q[IFO_QU]);
            flip_extrapolate(s, &s->q[IFO_QV]);
            break;
        }
        q_extrapolate(s, &s->q[IFO_QD]);
        q_extrapolate(s, &s->q[IFO_QU]);
        q_extrapolate(s, &s->q[IFO_QV]);
        break;
    case IFO_PH_P2G: if (v == IFO_FLIP) particles_to_grid(s); break;
    case IFO_PH_FLIP_COPY: if (v == IFO_FLIP) flip_copy(s); break;
    case IFO_PH_G2P: if (v == IFO_FLIP) flip_g2p(s); break;
    case IFO_PH_PADVECT: if (v == IFO_FLIP) particle_advect(s, dt); break;
    case IFO_PH_ADVECT:
        if (v == IFO_FLIP) break;
        q_advect(s, &s->q[IFO_QD], dt);
        if (v >= IFO_HEAT) q_advect(s, &s->q[IFO_QT], dt);
        q_advect(s, &s->q[IFO_QU], dt);
        q_advect(s, &s->q[IFO_QV], dt);
        for (int i = 0; i < 4; i++)
            if (s->q[i].present) flip(&s->q[i]);
        break;
    default: break;
    }
}

/* FluidSolver::update: 1-matrixless/Fluid.cpp:284-297, 3-conjugate-gradients/Fluid.cpp:433-447,
 * 4-solid-boundaries/Fluid.cpp:869-895, 5-curved-boundaries/Fluid.cpp:927-953,
 * 6-heat/Fluid.cpp:966-1006, 7-variable-density/Fluid.cpp:995-1034 */
void ifo_update(ifo_solver *s, double dt) {
    if (s->variant <= IFO_GS) {  /* 1-matrixless/Fluid.cpp:284-297 */
        ifo_phase(s, IFO_PH_RHS, dt);
        ifo_phase(s, IFO_PH_PROJECT, dt);
        ifo_phase(s, IFO_PH_APPLY_P, dt);
        ifo_phase(s, IFO_PH_ADVECT, dt);
        return;
    }
    if (s->variant == IFO_PLAIN) {
        ifo_phase(s, IFO_PH_RHS, dt);
        ifo_phase(s, IFO_PH_MATRIX, dt);
        ifo_phase(s, IFO_PH_PRECON, dt);
        ifo_phase(s, IFO_PH_PROJECT, dt);
        ifo_phase(s, IFO_PH_APPLY_P, dt);
        ifo_phase(s, IFO_PH_ADVECT, dt);
        return;
    }
    if (s->variant == IFO_FLIP) {  /* 8-flip/Fluid.cpp:1350-1413 */
        static const int order[] = {
            IFO_PH_FILL_SOLID, IFO_PH_P2G, IFO_PH_FLIP_COPY, IFO_PH_HEAT, IFO_PH_EXTRAP_T,
            IFO_PH_BUOYANCY, IFO_PH_BC, IFO_PH_RHS, IFO_PH_DENSITIES, IFO_PH_MATRIX,
            IFO_PH_PRECON, IFO_PH_PROJECT, IFO_PH_APPLY_P, IFO_PH_EXTRAP_DUV, IFO_PH_BC,
            IFO_PH_G2P, IFO_PH_PADVECT};
        for (size_t k = 0; k < sizeof order / sizeof order[0]; k++) ifo_phase(s, order[k], dt);
        return;
    }
    ifo_phase(s, IFO_PH_FILL_SOLID, dt);
    if (s->variant >= IFO_HEAT) {
        ifo_phase(s, IFO_PH_HEAT, dt);
        ifo_phase(s, IFO_PH_EXTRAP_T, dt);
        ifo_phase(s, IFO_PH_BUOYANCY, dt);
    }
    ifo_phase(s, IFO_PH_BC, dt);
    ifo_phase(s, IFO_PH_RHS, dt);
    ifo_phase(s, IFO_PH_DENSITIES, dt);
    ifo_phase(s, IFO_PH_MATRIX, dt);
    ifo_phase(s, IFO_PH_PRECON, dt);
    ifo_phase(s, IFO_PH_PROJECT, dt);
    ifo_phase(s, IFO_PH_APPLY_P, dt);
    ifo_phase(s, IFO_PH_EXTRAP_DUV, dt);
    ifo_phase(s, IFO_PH_BC, dt);
    ifo_phase(s, IFO_PH_ADVECT, dt);
}

void ifo_set_pinned_iterations(ifo_solver *s, int pressure, int heat) {
    s->pinned = pressure;
    s->pinned_heat = heat;
}

void ifo_get_stats(const ifo_solver *s, ifo_pcg_stats *pressure, ifo_pcg_stats *heat) {
    if (pressure) *pressure = s->st_pressure;
    if (heat) *heat = s->st_heat;
}

double *ifo_array(ifo_solver *s, int quantity_id, int which, int *w, int *h) {
    if (which >= IFO_A_R) {
        *w = s->w;
        *h = s->h;
        switch (which) {
        case IFO_A_R: return s->r;
        case IFO_A_P: return s->p;
        case IFO_A_Z: return s->z;
        case IFO_A_S: return s->s;
        case IFO_A_PRECON: return s->precon;
        case IFO_A_ADIAG: return s->adiag;
        case IFO_A_APLUSX: return s->aplusx;
        case IFO_A_APLUSY: return s->aplusy;
        case IFO_A_UDENS: *w = s->w + 1; return s->udens;
        case IFO_A_VDENS: *h = s->h + 1; return s->vdens;
        default: return NULL;
        }
    }
    if (quantity_id < 0 || quantity_id > 3 || !s->q[quantity_id].present) return NULL;
    quantity *q = &s->q[quantity_id];
    *w = q->w;
    *h = q->h;
    switch (which) {
    case IFO_A_SRC: return q->src;
    case IFO_A_DST: return q->dst;
    case IFO_A_PHI: *w = q->w + 1; *h = q->h + 1; return q->phi;
    case IFO_A_VOLUME: return q->volume;
    case IFO_A_NORMALX: return q->nx;
    case IFO_A_NORMALY: return q->ny;
    default: return NULL;
    }
}

uint8_t *ifo_bytes(ifo_solver *s, int quantity_id, int which, int *w, int *h) {
    if (quantity_id < 0 || quantity_id > 3 || !s->q[quantity_id].present) return NULL;
    quantity *q = &s->q[quantity_id];
    *w = q->w;
    *h = q->h;
    switch (which) {
    case IFO_B_CELL: return q->cell;
    case IFO_B_BODY: return q->body;
    case IFO_B_MASK: return q->mask;
    default: return NULL;
    }
}

void ifo_flip(ifo_solver *s, int quantity_id) {
    if (quantity_id >= 0 && quantity_id < 4 && s->q[quantity_id].present) flip(&s->q[quantity_id]);
}

/* toImage of each step (references in the header). */
void ifo_to_image(const ifo_solver *s, unsigned char *rgba, int heat) {
    const int w = s->w, h = s->h;
    const quantity *d = &s->q[0];
    if (s->variant <= 5) {
        for (int i = 0; i < w * h; i++) {
            int shade;
            if (s->variant == 5) shade = (int)((1.0 - d->src[i]) * d->volume[i] * 255.0);
            else shade = (int)((1.0 - d->src[i]) * 255.0);
            shade = shade < 255 ? shade : 255;  /* max(min(shade, 255), 0) */
            shade = shade < 0 ? 0 : shade;
            if (s->variant == 4 && d->cell[i] == CELL_SOLID) shade = 0;
            rgba[i * 4 + 0] = rgba[i * 4 + 1] = rgba[i * 4 + 2] = (unsigned char)shade;
            rgba[i * 4 + 3] = 0xFF;
        }
        return;
    }
    const quantity *t = &s->q[1];
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            const int idxl = 4 * (x + y * w * 2), idxr = heat ? 4 * (x + y * w * 2 + w) : 4 * (x + y * w);
            const double volume = d->volume[x + y * w];
            double shade = (1.0 - d->src[x + y * w]) * volume;
            shade = smin(smax(shade, 0.0), 1.0);
            rgba[idxr + 0] = rgba[idxr + 1] = rgba[idxr + 2] = (unsigned char)(int)(shade * 255.0);
            rgba[idxr + 3] = 0xFF;
            if (s->variant == IFO_FLIP && d->cell[x + y * w] == CELL_EMPTY) {
                rgba[idxr + 0] = 0xFF;
                rgba[idxr + 1] = rgba[idxr + 2] = 0;
            }
            if (heat) {
                double tt = s->variant == IFO_FLIP ? fabs(t->src[x + y * w] - s->t_amb) / 70.0
                                                   : (t->src[x + y * w] - s->t_amb) / 700.0;
                tt = smin(smax(tt, 0.0), 1.0);
                const double r = 1.0 + volume * (smin(tt * 4.0, 1.0) - 1.0);
                const double g = 1.0 + volume * (smin(tt * 2.0, 1.0) - 1.0);
                const double b = 1.0 + volume * (smax(smin(tt * 4.0 - 3.0, 1.0), 0.0) - 1.0);
                rgba[idxl + 0] = (unsigned char)(int)(r * 255.0);
                rgba[idxl + 1] = (unsigned char)(int)(g * 255.0);
                rgba[idxl + 2] = (unsigned char)(int)(b * 255.0);
                rgba[idxl + 3] = 0xFF;
            }
        }
    }
}

/* Scalar kernels exported for the known-answer tests. */
double ifo_occupancy(double d11, double d12, double d21, double d22) { return occupancy(d11, d12, d21, d22); }
double ifo_cerp(double a, double b, double c, double d, double x) { return cerp1(a, b, c, d, x); }
