/*
 * ifl_oracle.h - CPU oracle for the incremental-fluids per-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * solver's arithmetic (tunabrain/incremental-fluids, tutorial steps 1-8), used
 * by the tests as the parity checker and by bench.py as the timed CPU
 * baseline.  The CUDA product path never links, loads or calls it.
 *
 * Every array is FP64 and row-major (idx = x + y*w, no padding), exactly as in
 * the reference.  All buffers start zeroed (the reference leaves several
 * `new double[]` buffers uninitialised; both sides zero them so that
 * comparisons are defined).
 *
 * Parity is pinned bit-for-bit against the reference's own sources compiled
 * in place (oracle/ref_shim.cpp, built into oracle/_ref/ by oracle/Makefile).
 */
#ifndef IFL_ORACLE_H
#define IFL_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Variant = reference tutorial step whose FluidSolver::update is restated. */
enum {
    IFO_GS_EULER = 1, /* 1-matrixless: Gauss-Seidel solve, forward Euler + bilinear
                         advection, flat inflow                              */
    IFO_GS = 2,       /* 2-better-advection: Gauss-Seidel solve, step 3's
                         advection and inflow                                */
    IFO_PLAIN = 3,    /* 3-conjugate-gradients */
    IFO_SOLID = 4,    /* 4-solid-boundaries    */
    IFO_CURVED = 5,   /* 5-curved-boundaries   */
    IFO_HEAT = 6,     /* 6-heat                */
    IFO_VARDENS = 7,  /* 7-variable-density    */
    IFO_FLIP = 8      /* 8-flip: step 7's grid solve, FLIP particles carry
                         d, T, u, v instead of semi-Lagrangian advection */
};

/* Quantities (FluidQuantity instances). */
enum { IFO_QD = 0, IFO_QT = 1, IFO_QU = 2, IFO_QV = 3 };

/* Array identifiers for ifo_array(). */
enum {
    IFO_A_SRC = 0, IFO_A_DST = 1, IFO_A_PHI = 2, IFO_A_VOLUME = 3,
    IFO_A_NORMALX = 4, IFO_A_NORMALY = 5,
    /* solver-level arrays (quantity argument ignored) */
    IFO_A_R = 16, IFO_A_P = 17, IFO_A_Z = 18, IFO_A_S = 19,
    IFO_A_PRECON = 20, IFO_A_ADIAG = 21, IFO_A_APLUSX = 22, IFO_A_APLUSY = 23,
    IFO_A_UDENS = 24, IFO_A_VDENS = 25
};
enum { IFO_B_CELL = 0, IFO_B_BODY = 1, IFO_B_MASK = 2 };

/* Phases of FluidSolver::update, callable one at a time. */
enum {
    IFO_PH_FILL_SOLID = 0,   /* fillSolidFields on every quantity          */
    IFO_PH_HEAT = 1,         /* r=T, heat matrix, MIC(0), PCG, T=p          */
    IFO_PH_EXTRAP_T = 2,     /* _t->extrapolate()                           */
    IFO_PH_BUOYANCY = 3,     /* addBuoyancy                                 */
    IFO_PH_BC = 4,           /* setBoundaryCondition                        */
    IFO_PH_RHS = 5,          /* buildRhs                                    */
    IFO_PH_DENSITIES = 6,    /* computeDensities                            */
    IFO_PH_MATRIX = 7,       /* buildPressureMatrix                         */
    IFO_PH_PRECON = 8,       /* buildPreconditioner                         */
    IFO_PH_PROJECT = 9,      /* project(limit)                              */
    IFO_PH_APPLY_P = 10,     /* applyPressure                               */
    IFO_PH_EXTRAP_DUV = 11,  /* _d/_u/_v->extrapolate()                     */
    IFO_PH_ADVECT = 12,      /* advect every quantity, then flip           */
    /* step 8 (FLIP) only */
    IFO_PH_P2G = 13,         /* particlesToGrid: transfer, extrapolate,
                                count, prune, seed (initialises the
                                particles first when needed)               */
    IFO_PH_FLIP_COPY = 14,   /* copy() of every quantity, then the inflows
                                registered since the last update            */
    IFO_PH_G2P = 15,         /* diff, gridToParticles(alpha), undiff        */
    IFO_PH_PADVECT = 16      /* ParticleQuantities::advect                  */
};

/* Particle arrays of step 8 (ifo_particles). */
enum { IFO_P_X = 0, IFO_P_Y = 1, IFO_P_D = 2, IFO_P_T = 3, IFO_P_U = 4, IFO_P_V = 5 };

/* Solve outcome (the PCG of steps 3-8; the Gauss-Seidel solve of steps 1-2
 * reports sweeps made, CONVERGED or CAP, and the last maximum change). */
enum { IFO_PCG_CONVERGED = 0, IFO_PCG_INITIAL = 1, IFO_PCG_CAP = 2 };

typedef struct ifo_solver ifo_solver;

/* Body types: 0 = SolidBox, 1 = SolidSphere. */
typedef struct {
    int32_t type;
    int32_t pad_;
    double pos_x, pos_y, scale_x, scale_y, theta, vel_x, vel_y, vel_theta;
} ifo_body;

typedef struct {
    int32_t iterations;   /* matrix-vector products performed            */
    int32_t status;       /* IFO_PCG_*                                   */
    double max_error;     /* last infinity norm of the residual          */
} ifo_pcg_stats;

ifo_solver *ifo_create(int variant, int w, int h, double density_air,
                       double density_soot, double diffusion);
void ifo_destroy(ifo_solver *s);
int ifo_set_bodies(ifo_solver *s, const ifo_body *bodies, int n);
void ifo_get_bodies(const ifo_solver *s, ifo_body *bodies);
void ifo_advance_bodies(ifo_solver *s, double dt);
void ifo_add_inflow(ifo_solver *s, double x, double y, double w, double h,
                    double d, double t, double u, double v);
void ifo_update(ifo_solver *s, double dt);
void ifo_phase(ifo_solver *s, int phase, double dt);
/* -1: stop on the 1e-5 residual test (the reference); k >= 0: run exactly k
 * iterations (pinned mode, for separating rounding drift from a flip of the
 * termination test). */
void ifo_set_pinned_iterations(ifo_solver *s, int pressure, int heat);
void ifo_get_stats(const ifo_solver *s, ifo_pcg_stats *pressure, ifo_pcg_stats *heat);

/* Direct access to internal arrays (for state upload / download in tests). */
double *ifo_array(ifo_solver *s, int quantity, int which, int *w, int *h);
uint8_t *ifo_bytes(ifo_solver *s, int quantity, int which, int *w, int *h);
/* Swap src/dst of one quantity (FluidQuantity::flip). */
void ifo_flip(ifo_solver *s, int quantity);

/* FluidSolver::toImage: 8-bit RGBA, w x h (heat and step >= 6: 2w x h, heat
 * colours left, shade right); 3-conjugate-gradients/Fluid.cpp:455-465,
 * 4-solid-boundaries/Fluid.cpp:903-916, 5-curved-boundaries/Fluid.cpp:961-972,
 * 7-variable-density/Fluid.cpp:1047-1081, 8-flip/Fluid.cpp:1426-1470; step 8
 * paints CELL_EMPTY density cells red and scales heat by |T - Tamb|/70. */
void ifo_to_image(const ifo_solver *s, unsigned char *rgba, int heat);

/* Step 8 (FLIP) particle state.  ifo_particles returns the array (capacity
 * 12*w*h) and the live count; ifo_flip_init places the initial particles
 * (initParticles + gridToParticles(1.0), 8-flip/Fluid.cpp:733-750,
 * 1307-1314) if that has not happened yet - the first update does it
 * otherwise.  The random stream is the reference's frand() LCG, one stream
 * per solver, starting at 0xBA5EBA11. */
double *ifo_particles(ifo_solver *s, int which, int *count);
void ifo_set_particle_count(ifo_solver *s, int n);
void ifo_flip_init(ifo_solver *s);
uint32_t ifo_rng_state(const ifo_solver *s);
void ifo_set_rng_state(ifo_solver *s, uint32_t state);
/* frand() of 8-flip/Fluid.cpp:38-46 on an explicit state (known-answer tests). */
float ifo_frand(uint32_t *state);

/* Scalar kernels for known-answer tests: occupancy() of
 * 7-variable-density/Fluid.cpp:68-102 and the clamped Catmull-Rom of
 * 3-conjugate-gradients/Fluid.cpp:55-69. */
double ifo_occupancy(double d11, double d12, double d21, double d22);
double ifo_cerp(double a, double b, double c, double d, double x);

#ifdef __cplusplus
}
#endif
#endif
