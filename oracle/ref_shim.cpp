/*
 * ref_shim.cpp - builds the UNMODIFIED reference solver (one tutorial step's
 * Fluid.cpp, included in place from the reference checkout) into a shared
 * library with a small C interface, so that tests can pin the oracle
 * restatement (ifl_oracle.c) bit-for-bit against the reference itself.
 *
 * TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile into oracle/_ref/
 * (git-ignored) with -O2 -ffp-contract=off; REF_STEP selects the step and
 * REF_FLUID_CPP names the reference source file.
 *
 * The reference keeps its state private and has no readback besides PNG
 * output, so the include is preceded by access-widening macros; `main` is
 * renamed so that it is compiled but never run, and `printf` is routed to a
 * hook that records the PCG outcome lines instead of printing them.
 */
#include <algorithm>
#include <cmath>
#include <math.h>
#include <stack>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <string>
#include <vector>

#include "lodepng.h"

extern "C" int ref_printf_hook(const char *fmt, ...);

#define class struct
#define private public
#define protected public
#define main reference_main
#define printf ref_printf_hook
#include REF_FLUID_CPP
#undef printf
#undef main
#undef protected
#undef private
#undef class

/* main() of the reference writes PNG frames; it is never called here. */
unsigned lodepng_encode32_file(const char *, const unsigned char *, unsigned, unsigned) { return 0; }

namespace {
struct pcg_record { int iterations; int status; double max_error; };
pcg_record g_log[8];
int g_nlog = 0;
int g_particle_count = -1;
}

/* Records "Exiting solver after %d iterations, maximum error is %f",
 * "Exceeded budget of %d iterations, ..." and "Initial guess sufficiently
 * small" in call order (heat solve first, then pressure, in steps 6-7). */
extern "C" int ref_printf_hook(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    if (strncmp(fmt, "Particle", 8) == 0) {  /* step 8's particlesToGrid report */
        g_particle_count = va_arg(ap, int);
        va_end(ap);
        return 0;
    }
    pcg_record rec = {0, 1, 0.0};
    if (strncmp(fmt, "Exiting", 7) == 0) {
        int it = va_arg(ap, int);
        double e = va_arg(ap, double);
        rec = {it + 1, 0, e};
    } else if (strncmp(fmt, "Exceeded", 8) == 0) {
        int lim = va_arg(ap, int);
        double e = va_arg(ap, double);
        rec = {lim, 2, e};
    }
    va_end(ap);
    if (g_nlog < 8) g_log[g_nlog++] = rec;
    return 0;
}

namespace {
struct RefScene {
#if REF_STEP >= 4
    std::vector<const SolidBody *> cbodies;
    std::vector<SolidBody *> bodies;
#endif
    FluidSolver *solver = nullptr;
    int w = 0, h = 0;
    double rho_air = 0, rho_soot = 0, diffusion = 0;
};

void zero(double *p, size_t n) { memset(p, 0, n * sizeof(double)); }

void zero_quantity(FluidQuantity *q) {
    size_t n = (size_t)q->_w * q->_h;
#if REF_STEP == 8
    zero(q->_old, n);
#else
    zero(q->_dst, n);
#endif
#if REF_STEP >= 4
    zero(q->_normalX, n);
    zero(q->_normalY, n);
    memset(q->_body, 0, n);
    memset(q->_mask, 0, n);
#endif
#if REF_STEP >= 5
    zero(q->_phi, (size_t)(q->_w + 1) * (q->_h + 1));
#endif
}
/* Constructs the reference solver.  Step 8's constructor seeds particles
 * against the body list, so there it runs on first use, after the bodies have
 * been added (the reference's main also creates the bodies first). */
void build(RefScene *s) {
    const int w = s->w, h = s->h;
    const double rho_air = s->rho_air, rho_soot = s->rho_soot, diffusion = s->diffusion;
#if REF_STEP <= 3
    (void)rho_soot; (void)diffusion;
    s->solver = new FluidSolver(w, h, rho_air);
#elif REF_STEP <= 5
    (void)rho_soot; (void)diffusion;
    s->solver = new FluidSolver(w, h, rho_air, s->cbodies);
#else
    s->solver = new FluidSolver(w, h, rho_air, rho_soot, diffusion, s->cbodies);
#endif
    FluidSolver *f = s->solver;
    size_t n = (size_t)w * h;
    zero_quantity(f->_d);
    zero_quantity(f->_u);
    zero_quantity(f->_v);
#if REF_STEP >= 6
    zero_quantity(f->_t);
#endif
    zero(f->_r, n);
#if REF_STEP >= 3
    zero(f->_p, n); zero(f->_z, n); zero(f->_s, n);
    zero(f->_precon, n); zero(f->_aDiag, n); zero(f->_aPlusX, n); zero(f->_aPlusY, n);
#endif
#if REF_STEP >= 7
    zero(f->_uDensity, (size_t)(w + 1) * h);
    zero(f->_vDensity, (size_t)w * (h + 1));
#endif
}

FluidSolver *solver_of(void *p) {
    RefScene *s = (RefScene *)p;
    if (!s->solver) build(s);
    return s->solver;
}
}  // namespace

extern "C" {

void *ref_create(int w, int h, double rho_air, double rho_soot, double diffusion) {
    RefScene *s = new RefScene();
    s->w = w;
    s->h = h;
    s->rho_air = rho_air;
    s->rho_soot = rho_soot;
    s->diffusion = diffusion;
#if REF_STEP != 8
    build(s);
#endif
    return s;
}

void ref_destroy(void *p) {
    RefScene *s = (RefScene *)p;
#if REF_STEP == 8
    /* ~FluidSolver of step 8 deletes the quantities twice (once itself, once
     * through ~ParticleQuantities); the solver is left allocated. */
    s->solver = nullptr;
#endif
    delete s->solver;
#if REF_STEP >= 4
    for (SolidBody *b : s->bodies) delete b;
#endif
    delete s;
}

int ref_step(void) { return REF_STEP; }

void ref_add_body(void *p, int type, double px, double py, double sx, double sy,
                  double th, double vx, double vy, double vth) {
#if REF_STEP >= 4
    RefScene *s = (RefScene *)p;
    SolidBody *b;
    if (type == 0) b = new SolidBox(px, py, sx, sy, th, vx, vy, vth);
    else b = new SolidSphere(px, py, sx, th, vx, vy, vth);
    s->bodies.push_back(b);
    s->cbodies.push_back(b);
#else
    (void)p; (void)type; (void)px; (void)py; (void)sx; (void)sy; (void)th; (void)vx; (void)vy; (void)vth;
#endif
}

void ref_get_body(void *p, int i, double *out8) {
#if REF_STEP >= 4
    RefScene *s = (RefScene *)p;
    SolidBody *b = s->bodies[i];
    double v[8] = {b->_posX, b->_posY, b->_scaleX, b->_scaleY, b->_theta, b->_velX, b->_velY, b->_velTheta};
    memcpy(out8, v, sizeof v);
#else
    (void)p; (void)i; (void)out8;
#endif
}

void ref_advance_bodies(void *p, double dt) {
#if REF_STEP >= 4
    RefScene *s = (RefScene *)p;
    for (SolidBody *b : s->bodies) b->update(dt);
#else
    (void)p; (void)dt;
#endif
}

void ref_add_inflow(void *p, double x, double y, double w, double h, double d, double t, double u, double v) {
    RefScene *s = (RefScene *)p;
#if REF_STEP == 8
    /* step 8's update() applies its own fixed inflow (8-flip/Fluid.cpp:1368) */
    (void)s; (void)x; (void)y; (void)w; (void)h; (void)d; (void)t; (void)u; (void)v;
#elif REF_STEP >= 6
    s->solver->addInflow(x, y, w, h, d, t, u, v);
#else
    (void)t;
    s->solver->addInflow(x, y, w, h, d, u, v);
#endif
}

/* Runs FluidSolver::update; returns how many PCG outcomes were recorded. */
int ref_update(void *p, double dt) {
    RefScene *s = (RefScene *)p;
    g_nlog = 0;
    solver_of(s)->update(dt);
    return g_nlog;
}

/* k-th PCG outcome of the last update: iterations, status (0 converged,
 * 1 initial residual small enough, 2 iteration cap), last max error. */
int ref_pcg_record(int k, int *iterations, int *status, double *max_error) {
    if (k < 0 || k >= g_nlog) return -1;
    *iterations = g_log[k].iterations;
    *status = g_log[k].status;
    *max_error = g_log[k].max_error;
    return 0;
}

/* Same array identifiers as the oracle (ifl_oracle.h). */
double *ref_array(void *p, int qid, int which, int *w, int *h) {
    RefScene *s = (RefScene *)p;
    FluidSolver *f = solver_of(s);
    if (which >= 16) {
        *w = s->w;
        *h = s->h;
        switch (which) {
        case 16: return f->_r;
        case 17: return f->_p;
#if REF_STEP >= 3
        case 18: return f->_z;
        case 19: return f->_s;
        case 20: return f->_precon;
        case 21: return f->_aDiag;
        case 22: return f->_aPlusX;
        case 23: return f->_aPlusY;
#endif
#if REF_STEP >= 7
        case 24: *w = s->w + 1; return f->_uDensity;
        case 25: *h = s->h + 1; return f->_vDensity;
#endif
        default: return nullptr;
        }
    }
    FluidQuantity *q = nullptr;
    switch (qid) {
    case 0: q = f->_d; break;
#if REF_STEP >= 6
    case 1: q = f->_t; break;
#endif
    case 2: q = f->_u; break;
    case 3: q = f->_v; break;
    default: return nullptr;
    }
    *w = q->_w;
    *h = q->_h;
    switch (which) {
    case 0: return q->_src;
#if REF_STEP == 8
    case 1: return q->_old;
#else
    case 1: return q->_dst;
#endif
#if REF_STEP >= 5
    case 2: *w = q->_w + 1; *h = q->_h + 1; return q->_phi;
    case 3: return q->_volume;
#endif
#if REF_STEP >= 4
    case 4: return q->_normalX;
    case 5: return q->_normalY;
#endif
    default: return nullptr;
    }
}

uint8_t *ref_bytes(void *p, int qid, int which, int *w, int *h) {
#if REF_STEP >= 4
    RefScene *s = (RefScene *)p;
    FluidSolver *f = solver_of(s);
    FluidQuantity *q = nullptr;
    switch (qid) {
    case 0: q = f->_d; break;
#if REF_STEP >= 6
    case 1: q = f->_t; break;
#endif
    case 2: q = f->_u; break;
    case 3: q = f->_v; break;
    default: return nullptr;
    }
    *w = q->_w;
    *h = q->_h;
    switch (which) {
    case 0: return q->_cell;
    case 1: return q->_body;
    case 2: return q->_mask;
    default: return nullptr;
    }
#else
    (void)p; (void)qid; (void)which; (void)w; (void)h;
    return nullptr;
#endif
}

void ref_to_image(void *p, unsigned char *rgba, int heat) {
#if REF_STEP >= 6
    solver_of(p)->toImage(rgba, heat != 0);
#else
    (void)heat;
    ((RefScene *)p)->solver->toImage(rgba);
#endif
}

/* Step 8 particle arrays (ParticleQuantities::_posX, _posY, _properties[k])
 * and the live count; the same identifiers as ifo_particles. */
double *ref_particles(void *p, int which, int *count) {
#if REF_STEP == 8
    ParticleQuantities *q = solver_of(p)->_qs;
    *count = q->_particleCount;
    if (which == 0) return q->_posX;
    if (which == 1) return q->_posY;
    if (which >= 2 && which < 6) return q->_properties[which - 2];
    return nullptr;
#else
    (void)p; (void)which;
    *count = 0;
    return nullptr;
#endif
}

/* Sets the live particle count (tests write the arrays through ref_particles). */
void ref_set_particle_count(void *p, int n) {
#if REF_STEP == 8
    solver_of(p)->_qs->_particleCount = n;
#else
    (void)p; (void)n;
#endif
}

/* Particle count the last particlesToGrid printed (-1 before any). */
int ref_particle_report(void) { return g_particle_count; }

}  // extern "C"
