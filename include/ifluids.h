/*
 * ifluids.h - C ABI of the GB300 (sm_103a) incremental-fluids solver.
 *
 * One handle = one FluidSolver of the reference (tunabrain/incremental-fluids),
 * with its state resident in device memory.  The handle owns every device
 * buffer; the caller owns host buffers.  All calls on one handle must come from
 * one host thread at a time; distinct handles may be driven from distinct
 * threads.  Work is enqueued on the handle's CUDA stream; calls that return
 * data to the host synchronise that stream.  No exception crosses this ABI:
 * every entry point returns an ifl_status.
 *
 * Reference surface replaced (paths inside the reference project):
 *   FluidSolver(int w, int h, double density)            3-conjugate-gradients/Fluid.cpp:401
 *   FluidSolver(w, h, density, bodies)                   4-solid-boundaries/Fluid.cpp:836,
 *                                                        5-curved-boundaries/Fluid.cpp:894
 *   FluidSolver(w, h, rhoAir, rhoSoot, diffusion, bodies) 6-heat/Fluid.cpp:921,
 *                                                        7-variable-density/Fluid.cpp:945
 *   void addInflow(x, y, w, h, d, u, v)                  3-conjugate-gradients/Fluid.cpp:449
 *   void addInflow(x, y, w, h, d, t, u, v)               7-variable-density/Fluid.cpp:1036
 *   void update(double timestep)                         3-conjugate-gradients/Fluid.cpp:433,
 *                                                        7-variable-density/Fluid.cpp:995
 *   double ambientT()                                    7-variable-density/Fluid.cpp:1043
 *   SolidBox / SolidSphere / SolidBody::update           4-solid-boundaries/Fluid.cpp:79-241
 * The reference has no field readback (only toImage -> PNG); ifl_read_field
 * is the replacement for that.
 */
#ifndef IFLUIDS_H
#define IFLUIDS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ifl_solver ifl_solver;

/* Status codes. */
enum {
    IFL_OK = 0,
    IFL_ERR_ARG = -1,        /* invalid argument                                  */
    IFL_ERR_CUDA = -2,       /* CUDA runtime error (see ifl_last_error)           */
    IFL_ERR_NOMEM = -3,      /* device allocation failed                          */
    IFL_ERR_TIMEOUT = -4,    /* a bounded device-side wait gave up (status word)  */
    IFL_ERR_UNSUPPORTED = -5 /* configuration outside the supported envelope      */
};

/* Variant = tutorial step of the reference whose update() is reproduced. */
enum {
    IFL_GS_EULER = 1, /* 1-matrixless: Gauss-Seidel solve, forward Euler +
                         bilinear advection, flat inflow (h <= 1024)          */
    IFL_GS = 2,       /* 2-better-advection: Gauss-Seidel solve, step 3's
                         advection and inflow (h <= 1024)                     */
    IFL_PLAIN = 3,    /* 3-conjugate-gradients: MIC(0)-PCG, no solids          */
    IFL_SOLID = 4,    /* 4-solid-boundaries: binary solid cells               */
    IFL_CURVED = 5,   /* 5-curved-boundaries: fractional cell volumes         */
    IFL_HEAT = 6,     /* 6-heat: + temperature, heat diffusion, buoyancy       */
    IFL_VARDENS = 7,  /* 7-variable-density: + per-face density               */
    IFL_FLIP = 8      /* 8-flip: step 7's grid solve; FLIP particles carry d,
                         T, u, v instead of semi-Lagrangian advection.  Fields
                         and particles are FP64 in both forms; IFL_FP32 selects
                         FP32-form solves                                     */
};

/* Storage / arithmetic form. */
enum {
    IFL_FP64 = 0,  /* drop-in: FP64 everywhere, bit-exact advection/assembly   */
    IFL_FP32 = 1   /* FP32 fields, matrix, advection, matvec, MIC(0) apply;
                      FP64 dot products, max-norm, alpha/beta, MIC(0) factor */
};

/* Element types for field transfer. */
enum { IFL_DT_F64 = 0, IFL_DT_F32 = 1, IFL_DT_U8 = 2 };

/* Quantities. */
enum { IFL_Q_D = 0, IFL_Q_T = 1, IFL_Q_U = 2, IFL_Q_V = 3 };

/* Per-quantity arrays; a field id is IFL_FIELD(quantity, array). */
enum {
    IFL_A_SRC = 0,      /* the quantity itself (FluidQuantity::_src)            */
    IFL_A_DST = 1,      /* advection target buffer (FluidQuantity::_dst)        */
    IFL_A_PHI = 2,      /* distance samples at cell corners, (w+1) x (h+1)      */
    IFL_A_VOLUME = 3,   /* fluid volume fraction                                 */
    IFL_A_NORMALX = 4,
    IFL_A_NORMALY = 5,
    IFL_A_CELL = 8,     /* u8: 0 fluid, 1 solid, 2 empty (step 8, transient)    */
    IFL_A_BODY = 9      /* u8: index of the nearest body                         */
};
#define IFL_FIELD(q, a) (((q) << 8) | (a))
/* Solver-level arrays (w x h unless noted). */
enum {
    IFL_F_R = 16, IFL_F_P = 17, IFL_F_Z = 18, IFL_F_S = 19, IFL_F_PRECON = 20,
    IFL_F_ADIAG = 21, IFL_F_APLUSX = 22, IFL_F_APLUSY = 23,
    IFL_F_UDENS = 24,   /* (w+1) x h */
    IFL_F_VDENS = 25    /* w x (h+1) */
};

/* Phases of one update(), for per-phase parity runs (ifl_run_phase). */
enum {
    IFL_PH_FILL_SOLID = 0, IFL_PH_HEAT = 1, IFL_PH_EXTRAP_T = 2, IFL_PH_BUOYANCY = 3,
    IFL_PH_BC = 4, IFL_PH_RHS = 5, IFL_PH_DENSITIES = 6, IFL_PH_MATRIX = 7,
    IFL_PH_PRECON = 8, IFL_PH_PROJECT = 9, IFL_PH_APPLY_P = 10,
    IFL_PH_EXTRAP_DUV = 11, IFL_PH_ADVECT = 12,
    /* step 8 (FLIP) only */
    IFL_PH_P2G = 13,        /* particlesToGrid: transfer, extrapolation, count,
                               prune, seed (places the initial particles first
                               when that has not happened)                      */
    IFL_PH_FLIP_COPY = 14,  /* copy() of every quantity, then the inflows added
                               since the last update                            */
    IFL_PH_G2P = 15,        /* diff, gridToParticles(alpha), undiff             */
    IFL_PH_PADVECT = 16     /* ParticleQuantities::advect                      */
};

/* PCG outcome. */
enum { IFL_PCG_CONVERGED = 0, IFL_PCG_INITIAL = 1, IFL_PCG_CAP = 2 };

typedef struct {
    int32_t variant;           /* IFL_GS_EULER .. IFL_FLIP                       */
    int32_t w, h;              /* pressure grid size (>= 2 each)                 */
    int32_t precision;         /* IFL_FP64 or IFL_FP32                           */
    double density_air;        /* `density` of steps 3-5, rhoAir of 6-7 (0.1)    */
    double density_soot;       /* rhoSoot (1.0)                                  */
    double diffusion;          /* heat diffusion (0.01)                          */
    int32_t max_iter_pressure; /* 600 in steps 1-3 (Gauss-Seidel sweeps in 1-2),
                                  2000 in steps 4-8                             */
    int32_t max_iter_heat;     /* 2000                                           */
    void *stream;              /* cudaStream_t to use; NULL = handle-owned stream */
    int32_t device;            /* CUDA device ordinal the handle lives on (0)    */
    int32_t pad_;
} ifl_params;

/* Solid body; same parameters as SolidBox(x, y, sx, sy, t, vx, vy, vt) and
 * SolidSphere(x, y, s, t, vx, vy, vt) (scale_y is ignored for spheres). */
typedef struct {
    int32_t type;  /* 0 = box, 1 = sphere */
    int32_t pad_;
    double pos_x, pos_y, scale_x, scale_y, theta, vel_x, vel_y, vel_theta;
} ifl_body;

typedef struct {
    int32_t iterations;  /* matrix-vector products performed by the last solve */
    int32_t status;      /* IFL_PCG_*                                          */
    double max_error;    /* last infinity norm of the residual                 */
} ifl_pcg_stats;

typedef struct {
    ifl_pcg_stats pressure;
    ifl_pcg_stats heat;
    uint32_t device_flags;  /* bit 0: bounded wait timed out; bit 1: solid cell on
                               the outer ring (outside the parity envelope);
                               bit 2 (step 8): seeding tested a particle number
                               beyond the live count (fewer particles than
                               cells); bit 3: empty-cell extrapolation exceeded
                               its work bound */
    uint32_t steps;         /* update() calls completed                         */
} ifl_step_stats;

/* Fill *p with the reference's defaults for a variant and grid size. */
void ifl_default_params(ifl_params *p, int variant, int w, int h);

/* FluidSolver constructors (all steps). */
int ifl_create(const ifl_params *p, ifl_solver **out);
int ifl_destroy(ifl_solver *s);

/* Bodies (steps 4-8).  The reference keeps references to caller-owned bodies
 * and the caller moves them between steps (SolidBody::update); here the caller
 * passes the current body table before update() (it is copied), or lets the
 * handle advance its own copy with ifl_advance_bodies. */
int ifl_set_bodies(ifl_solver *s, const ifl_body *bodies, int n);
int ifl_get_bodies(ifl_solver *s, ifl_body *bodies, int capacity, int *n);
int ifl_advance_bodies(ifl_solver *s, double dt);

/* FluidSolver::addInflow; `t` is ignored below step 6.  Step 8 adds its
 * inflow inside update(), between copy() and the heat solve
 * (8-flip/Fluid.cpp:1365-1368): there the rectangles added before update()
 * are applied at that point of the next update. */
int ifl_add_inflow(ifl_solver *s, double x, double y, double w, double h,
                   double d, double t, double u, double v);
/* FluidSolver::update; asynchronous on the handle's stream. */
int ifl_update(ifl_solver *s, double dt);
/* Run one phase of update() (tests; same semantics as inside update). */
int ifl_run_phase(ifl_solver *s, int phase, double dt);
/* FluidSolver::ambientT (294 K). */
double ifl_ambient_t(const ifl_solver *s);

/* Field transfer between the device state and a dense row-major host array
 * (idx = x + y*w).  `dtype` converts on the fly.  Both synchronise. */
int ifl_field_shape(const ifl_solver *s, int field, int *w, int *h);
int ifl_read_field(ifl_solver *s, int field, void *host, size_t bytes, int dtype);
int ifl_write_field(ifl_solver *s, int field, const void *host, size_t bytes, int dtype);
/* FluidSolver::toImage (3-conjugate-gradients/Fluid.cpp:455-465,
 * 4-solid-boundaries/Fluid.cpp:903-916, 5-curved-boundaries/Fluid.cpp:961-972,
 * 7-variable-density/Fluid.cpp:1047-1081, 8-flip/Fluid.cpp:1426-1470): 8-bit RGBA, w x h pixels, pixel
 * (x, y) at 4*(x + y*width); with heat != 0 in steps 6-8 the image is 2w wide
 * (heat colours left, density shade right) as renderHeat in the reference.
 * on_device = 0: `rgba` is host memory and the call synchronises; 1: `rgba`
 * is device memory, written asynchronously on the handle's stream (a headless
 * frame for GPU-side consumers).  The reference encodes PNGs with lodepng;
 * the Python package writes them (ifluids.write_png). */
int ifl_render(ifl_solver *s, int heat, void *rgba, size_t bytes, int on_device);
/* FluidQuantity::flip for one quantity (tests). */
int ifl_flip(ifl_solver *s, int quantity);

/* Step 8 (FLIP) particles: ParticleQuantities::_posX, _posY and the carried
 * d, T, u, v (8-flip/Fluid.cpp:692-722), FP64, capacity 12 per cell.  The
 * initial particles (initParticles + gridToParticles(1.0) of the
 * constructor, 8-flip/Fluid.cpp:733-750, 1307-1314) are placed by the first
 * update, against the bodies set by then, or by ifl_flip_init.  Reads and
 * writes synchronise.  Writing a count replaces the initial placement. */
enum { IFL_P_X = 0, IFL_P_Y = 1, IFL_P_D = 2, IFL_P_T = 3, IFL_P_U = 4, IFL_P_V = 5 };
int ifl_flip_init(ifl_solver *s);
int ifl_particle_count(ifl_solver *s, int *n);
int ifl_read_particles(ifl_solver *s, int which, double *out, int capacity, int *n);
int ifl_write_particles(ifl_solver *s, int which, const double *in, int n);
int ifl_set_particle_count(ifl_solver *s, int n);
/* frand() state (8-flip/Fluid.cpp:38-46), one stream per handle starting at
 * 0xBA5EBA11 as the reference's static seed. */
int ifl_get_rng_state(ifl_solver *s, uint32_t *state);
int ifl_set_rng_state(ifl_solver *s, uint32_t state);

/* PCG outcome of the last update (synchronises). */
int ifl_get_stats(ifl_solver *s, ifl_step_stats *out);
/* Per solve: -1 stops on the residual test (default); k >= 0 runs exactly k
 * iterations (separates rounding drift from a flip of the termination test). */
int ifl_set_pinned_iterations(ifl_solver *s, int pressure, int heat);

/* Failure detection: every device-side wait of a solve (a strip waiting for
 * its neighbour's boundary row, a team barrier, a Gauss-Seidel progress
 * counter) gives up after `polls` polls; the solve then runs to its end without
 * waiting, the handle's status word gets bit 0 and ifl_get_stats returns
 * IFL_ERR_TIMEOUT.  0 restores the default (about a second of polling).  A
 * batch waits with the limit of its first member.  No counterpart in the
 * reference, which has no device waits. */
int ifl_set_wait_limit(ifl_solver *s, int64_t polls);

/* Kernel timing.  When on, every kernel group launched by the handle is
 * bracketed by CUDA events on the handle's stream (no host synchronisation);
 * ifl_get_timing synchronises, returns the accumulated device time per group
 * and resets the accumulators. */
enum {
    IFL_K_PCG = 0,         /* persistent MIC(0)-PCG kernel (factor + solve)   */
    IFL_K_ASSEMBLE = 1,    /* RHS / densities / matrix / heat matrix          */
    IFL_K_ADVECT = 2,      /* fused advection of every quantity               */
    IFL_K_SOLID = 3,       /* distance field, cells, normals, volumes         */
    IFL_K_EXTRAPOLATE = 4, /* solid-cell extrapolation                        */
    IFL_K_FACES = 5,       /* inflow, boundary conditions, buoyancy, pressure update */
    IFL_K_PARTICLES = 6,   /* step 8: particle transfers, seeding, advection  */
    IFL_K_GROUPS = 7
};
typedef struct {
    double ms[IFL_K_GROUPS];           /* device time per group               */
    int64_t launches[IFL_K_GROUPS];    /* timed launches per group            */
    int64_t pcg_iterations;            /* PCG iterations inside the timed PCG launches */
} ifl_timing;
int ifl_set_timing(ifl_solver *s, int on);
int ifl_get_timing(ifl_solver *s, ifl_timing *out);

/* Pressure solve that allocates nothing.  This entry point has no counterpart
 * in the reference: it serves callers that cannot allocate device memory
 * while they run (code inside another framework's memory pool or under a
 * fixed memory budget, real-time loops that must not enter the allocator,
 * processes that forbid cudaMalloc after start-up).
 *
 * Solves the unmasked MIC(0)-preconditioned CG system of
 * 3-conjugate-gradients (buildPreconditioner + project) for a w x h grid:
 * adiag, aplusx, aplusy, rhs and p are DEVICE arrays, dense row-major
 * (idx = x + y*w), FP64; `stats` is a DEVICE ifl_pcg_stats the solve writes
 * its outcome into (status -1: a bounded device-side wait timed out).
 * Work is enqueued on `stream` (NULL: the default stream); nothing is
 * synchronised.
 *
 * Every intermediate array lives in one fixed device array inside the
 * library (about 8.4 MB, held by every GPU that loads the library until the
 * process exits).  Limit: the grid must fit 2304 strip-diagonals, i.e.
 * ceil(h/32) * round_up(w + 31, 16) <= 2304 (for example 256 x 256); larger
 * grids return IFL_ERR_UNSUPPORTED without touching the GPU.  It calls no
 * cudaMalloc, cudaFree or other allocating routine.  All calls share that
 * array, which keeps the last call's contents: calls whose work overlaps on
 * the GPU (different streams, or different host threads) race and must be
 * serialised by the caller.  The first call on each device looks up the
 * array's device address (cudaGetSymbolAddress) with that device current.
 * Under CUDA's lazy module loading (the default) that lookup is also when the
 * driver loads this library's device code and reserves the array on that
 * device, so a caller that must not allocate while it runs should make one
 * call per device at start-up (any grid, e.g. a 2 x 2 solve), and before any
 * stream capture. */
int ifl_pcg_solve_noalloc(int w, int h, const double *adiag, const double *aplusx,
                          const double *aplusy, const double *rhs, double *p, int max_iter,
                          ifl_pcg_stats *stats, void *stream);

/* ------------------------------------------------------------------ batches
 * Many independent scenes advanced together.  The reference runs one
 * FluidSolver per process and has no batch; a batch replaces a loop of
 * `solver.update(dt)` calls over many handles (3-conjugate-gradients/Fluid.cpp:433-447
 * ... 7-variable-density/Fluid.cpp:995-1034, once per handle) by one step of
 * batched launches: each phase runs for every scene in one launch and both
 * PCG solves of every scene run in one persistent cooperative launch whose
 * teams of blocks take scenes from work queues.  Results per scene equal
 * ifl_update on that handle (same arithmetic; FP64 sums of the PCG in a
 * different fixed order).
 *
 * Members are caller-owned handles of one device, variant and precision;
 * they must outlive the batch and must not be used by other threads during
 * ifl_batch_update.  Between batch steps each member remains a normal handle
 * (read fields, set bodies, ...). */
typedef struct ifl_batch ifl_batch;

/* One inflow rectangle with the arguments of FluidSolver::addInflow. */
typedef struct {
    double x, y, w, h, d, t, u, v;
} ifl_inflow;

typedef struct {
    /* Shape of the batched PCG launch: threads per block (32, 64, 128 or 256),
     * strips per block, bulk-copy ring stages.  threads = 0: autotune at the
     * first update (each candidate shape runs a few pinned PCG iterations of
     * the real system; the fastest is kept, unless the home shape, the first
     * candidate, is within 5 % of it: such a short trial cannot separate
     * closer shapes). */
    int32_t threads, strips_per_block, stages;
    int32_t use_graph;        /* 1: replay each step as one CUDA graph (default) */
    int32_t tune_iterations;  /* PCG iterations per autotuning trial (default 8) */
    int32_t max_team_blocks;  /* largest team (blocks working on one scene); 0: 128 */
    /* Tile shapes (threads x rows of one block) of the tiled phase kernels.
     * 1 (default): at the first update every candidate shape runs each phase
     * of IFL_TILE_FILL .. IFL_TILE_ADVECT twice on the real state (those
     * phases are idempotent) and the fastest is kept per phase; 0: 32 x 8
     * everywhere; 2: the shapes given in tile_w / tile_h.  A cell's results do
     * not depend on the tile shape. */
    int32_t tile_tune;
    int32_t pad_;
    int32_t tile_w[8], tile_h[8]; /* tile_tune 2: per IFL_TILE_* phase; one of the candidates */
} ifl_batch_options;

/* Tiled phases of a batch step (index into tile_w / tile_h). */
enum {
    IFL_TILE_FILL = 0,          /* fillSolidFields: phi, cell, volume, normals */
    IFL_TILE_BC = 1,            /* setBoundaryCondition */
    IFL_TILE_ASSEMBLE = 2,      /* buildRhs, buildPressureMatrix, densities */
    IFL_TILE_HEAT_ASSEMBLE = 3, /* heat matrix and right-hand side */
    IFL_TILE_ADVECT = 4,        /* advect of every quantity */
    IFL_TILE_APPLY = 5,         /* applyPressure (32 x 8: not idempotent, not tuned) */
    IFL_TILE_BUOYANCY = 6,      /* addBuoyancy (32 x 8, not tuned) */
    IFL_TILE_MASK = 7,          /* extrapolation mask (32 x 8, not tuned) */
    IFL_TILE_PHASES = 8
};
/* Candidate tile shapes (threads x rows): 32x8, 32x4, 64x4, 16x16, 128x2, 64x2. */

typedef struct {
    int32_t members;
    int32_t threads, strips_per_block, stages;  /* PCG shape in use            */
    int32_t grid;                               /* blocks of the PCG launch    */
    int32_t graph;                              /* 1: steps replay a CUDA graph */
    int32_t candidates;                         /* shapes tried by the autotuner */
    int32_t pad_;
    double candidate_ms[8];                     /* trial time of each candidate */
    double last_step_ms;                        /* device time of the last step */
    double last_pcg_ms;                         /* of which PCG launches        */
    int64_t launches;                           /* kernels launched by the batch */
    int64_t steps;
    int64_t h2d_bytes_last_step;                /* host -> device bytes of the last step */
    int64_t d2h_bytes_last_step;                /* device -> host bytes of the last step */
    int32_t tile_w[8], tile_h[8];               /* tile shape of each IFL_TILE_* phase in use */
    double tile_ms[8];                          /* tuned phases: trial time of the shape kept (ms) */
} ifl_batch_info;

void ifl_batch_default_options(ifl_batch_options *o);
int ifl_batch_create(ifl_solver *const *members, int n, const ifl_batch_options *opt, ifl_batch **out);
int ifl_batch_destroy(ifl_batch *b);
/* Inflows applied at the start of every batch step, in order (the batched
 * form of calling addInflow before each update); replaces the member's list. */
int ifl_batch_set_inflows(ifl_batch *b, int member, const ifl_inflow *rects, int n);
/* One update(dt) of every member; returns when the step has completed.  The
 * members' current body tables are used (see ifl_set_bodies). */
int ifl_batch_update(ifl_batch *b, double dt);
/* Per-member PCG outcome of the last batch step (n = member count). */
int ifl_batch_get_stats(ifl_batch *b, ifl_step_stats *out, int n);
int ifl_batch_get_info(ifl_batch *b, ifl_batch_info *out);
void *ifl_batch_stream(ifl_batch *b);
/* Host-only preview of how a batched PCG launch of `grid` blocks splits into
 * teams (no GPU work).  Scene i has strips[i] 32-row strips and estimated work
 * work[i]; it is solved by a team of the smallest power-of-two block count that
 * covers its strips.  teams[c] (c < 8) receives the number of teams of 2^c
 * blocks.  Returns the blocks placed in teams, or IFL_ERR_UNSUPPORTED when
 * the grid cannot hold one team of every size needed. */
int ifl_batch_plan_teams(int grid, int strips_per_block, int n, const int *strips, const double *work,
                         int *teams);
/* NULL: why the last ifl_batch_create on this thread failed. */
const char *ifl_batch_last_error(const ifl_batch *b);

/* ------------------------------------------------------------------ serving
 * Continuous batching of simulation requests (no counterpart in the
 * reference, which runs one scene per process).  A request is a scene (grid
 * size, bodies, inflow rectangles applied before every step) and a number of
 * update() calls.  ifl_server_step admits waiting requests in arrival order
 * while their device state fits the HBM budget and the member cap, then
 * advances every admitted request by one update() in one batch step (see
 * ifl_batch_update); requests that arrive while others run join at the next
 * step.  A finished request keeps its device state until ifl_server_release.
 * A request's results do not depend on the other requests in the batch
 * (bit-identical alone and in any mix).  Times are seconds on the server's
 * clock (ifl_server_now); `arrival` is supplied by the caller. */
typedef struct ifl_server ifl_server;

typedef struct {
    int32_t variant, precision, device;
    int32_t max_active;          /* scenes per batch step (default 1024)               */
    double dt;                   /* time step of every request (0.0025)                */
    int64_t hbm_budget_bytes;    /* device bytes for admitted requests; 0: no limit    */
    int32_t dry_run;             /* 1: bookkeeping only, no device work (planning, tests) */
    int32_t pad_;
    ifl_batch_options batch;     /* PCG shape (threads = 0: autotuned once, then kept) */
} ifl_server_params;

typedef struct {
    int32_t w, h, steps, n_bodies, n_inflows, pad_;
    const ifl_body *bodies;
    const ifl_inflow *inflows;
    double arrival;
} ifl_request;

typedef struct {
    int64_t id;
    int32_t w, h, steps, pad_;
    double arrival, admitted, finished;
    int64_t device_bytes;
} ifl_completion;

typedef struct {
    int32_t active, queued;
    int64_t bytes_in_use, cell_steps, steps, rebuilds;
    int32_t threads, strips_per_block, stages, pad_;
    int64_t peak_queued;  /* longest queue seen at a step (after admission)     */
    int64_t admitted, completed;  /* requests admitted / finished so far         */
    double rebuild_ms;    /* host time spent on new memberships: building the
                             batch and what its first step costs beyond a
                             steady step (plan, graph capture)               */
} ifl_server_info;

void ifl_server_default_params(ifl_server_params *p, int variant, int precision);
int ifl_server_create(const ifl_server_params *p, ifl_server **out);
int ifl_server_destroy(ifl_server *s);
double ifl_server_now(const ifl_server *s);
/* Queue a request; IFL_ERR_NOMEM when it alone exceeds the budget. */
int ifl_server_submit(ifl_server *s, const ifl_request *r, int64_t *id);
/* Admit, then one update() of every admitted request; returns when done. */
int ifl_server_step(ifl_server *s, int *active, int *queued);
/* Requests finished since the last call, in finishing order. */
int ifl_server_completions(ifl_server *s, ifl_completion *out, int capacity, int *n);
int ifl_server_field_shape(ifl_server *s, int64_t id, int field, int *w, int *h);
int ifl_server_read_field(ifl_server *s, int64_t id, int field, void *host, size_t bytes, int dtype);
int ifl_server_request_stats(ifl_server *s, int64_t id, ifl_step_stats *out);
int ifl_server_release(ifl_server *s, int64_t id);
int ifl_server_get_info(const ifl_server *s, ifl_server_info *out);
const char *ifl_server_last_error(const ifl_server *s);
/* Device bytes ifl_create allocates for these parameters (no GPU work). */
int64_t ifl_device_bytes(const ifl_params *p);

int ifl_synchronize(ifl_solver *s);
void *ifl_stream(ifl_solver *s);
/* Kernel launches of this library issued by the handle since creation. */
int64_t ifl_launch_count(const ifl_solver *s);
const char *ifl_last_error(const ifl_solver *s);
const char *ifl_version(void);

#ifdef __cplusplus
}
#endif
#endif
