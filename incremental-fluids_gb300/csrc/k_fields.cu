// k_fields.cu - per-cell / per-face kernels of one solver step (sm_103a).
//
// Each kernel is a gather: one thread owns one output cell or face and
// reproduces, in the same floating-point order, every update the reference's
// row-major loops apply to that location (scatters such as applyPressure and
// setBoundaryCondition become "earlier cell first" gathers).  FP64 storage
// gives results identical to the reference; FP32 storage runs the same
// formulas (advection in FP32, cheap per-cell bookkeeping in FP64 then
// rounded).
#include "ifl_device.cuh"

namespace ifl {

namespace {

__device__ __forceinline__ int qid_of(int nq, int z) { return nq == 4 ? z : (z == 0 ? 0 : z + 1); }

template <typename F> __device__ __forceinline__ F ldv(const F *p) { return *(const volatile F *)p; }
template <typename F> __device__ __forceinline__ void stv(F *p, F v) { *(volatile F *)p = v; }

// ----------------------------------------------------------------- inflow
// FluidQuantity::addInflow (3-conjugate-gradients/Fluid.cpp:167-184; step 1
// sets the value itself without the pulse, 1-matrixless/Fluid.cpp:141-151).  The x
// bound is the quantity's height (as in the reference) and cells are
// addressed by the flat index x + y*w.  When that index can wrap into the next
// row two rectangle cells may hit one location, so the rectangle is then
// walked by one thread in the reference's order.
template <typename F>
__device__ __forceinline__ void inflow_body(const Quant<F> &Q, int P, double hx, double x0, double y0, double x1,
                                            double y1, double val, bool flat = false) {
    int ix0 = (int)(x0 / hx - Q.ox);
    int iy0 = (int)(y0 / hx - Q.oy);
    int ix1 = (int)(x1 / hx - Q.ox);
    int iy1 = (int)(y1 / hx - Q.oy);
    int ylo = max(iy0, 0), yhi = min(iy1, Q.h);
    int xlo = max(ix0, 0), xhi = min(ix1, Q.h);
    if (ylo >= yhi || xlo >= xhi) return;
    long n = (long)Q.w * Q.h;
    int nx = xhi - xlo, ncell = nx * (yhi - ylo);
    bool serial = xhi > Q.w;
    int start = serial ? 0 : threadIdx.x;
    int step = serial ? 1 : blockDim.x;
    if (serial && threadIdx.x != 0) return;
    for (int i = start; i < ncell; i += step) {
        int x = xlo + i % nx, y = ylo + i / nx;
        double l = length2((2.0 * (x + 0.5) * hx - (x0 + x1)) / (x1 - x0),
                           (2.0 * (y + 0.5) * hx - (y0 + y1)) / (y1 - y0));
        double vi = flat ? val : cubic_pulse(l) * val;
        long flat = (long)x + (long)y * Q.w;
        if (flat >= n) continue;
        int fx = (int)(flat % Q.w), fy = (int)(flat / Q.w);
        F *c = Q.src + fx + (size_t)fy * P;
        if (fabs((double)*c) < fabs(vi)) *c = (F)vi;
    }
}
template <typename F>
__global__ void inflow_kernel(Quant<F> Q, int P, double hx, double x0, double y0, double x1, double y1,
                              double val, bool flat) {
    inflow_body(Q, P, hx, x0, y0, x1, y1, val, flat);
}

// ------------------------------------------------------------ solid fields
// fillSolidFields, distance grid part (7-variable-density/Fluid.cpp:479-488)
template <typename F>
__device__ __forceinline__ void phi_body(const Scene<F> &S, const uint3 bid) {
    Quant<F> Q = S.q[qid_of(S.nq, bid.z)];
    int ix = bid.x * blockDim.x + threadIdx.x, iy = bid.y * blockDim.y + threadIdx.y;
    if (ix > Q.w || iy > Q.h) return;
    double x = (ix + Q.ox - 0.5) * S.hx;
    double y = (iy + Q.oy - 0.5) * S.hx;
    double phi = body_distance(S.bodies[0], x, y);
    for (int i = 1; i < S.nbodies; i++) phi = smin(phi, body_distance(S.bodies[i], x, y));
    Q.phi[ix + (size_t)iy * S.P] = phi;
}
template <typename F>
__global__ void phi_kernel(Scene<F> S) { phi_body(S, blockIdx); }

// fillSolidFields, per-cell part (4-solid-boundaries/Fluid.cpp:453-479,
// 7-variable-density/Fluid.cpp:490-521)
template <typename F>
__device__ __forceinline__ void cell_body(const Scene<F> &S, const uint3 bid) {
    Quant<F> Q = S.q[qid_of(S.nq, bid.z)];
    int ix = bid.x * blockDim.x + threadIdx.x, iy = bid.y * blockDim.y + threadIdx.y;
    if (ix >= Q.w || iy >= Q.h) return;
    size_t idx = ix + (size_t)iy * S.P;
    double x = (ix + Q.ox) * S.hx;
    double y = (iy + Q.oy) * S.hx;
    int body = 0;
    double d = body_distance(S.bodies[0], x, y);
    for (int i = 1; i < S.nbodies; i++) {
        double id = body_distance(S.bodies[i], x, y);
        if (id < d) {
            body = i;
            d = id;
        }
    }
    Q.body[idx] = (uint8_t)body;
    uint8_t cell;
    double nx, ny;
    if (S.variant >= 5) {
        double vol = 1.0 - occupancy(Q.phi[idx], Q.phi[idx + 1], Q.phi[idx + S.P], Q.phi[idx + S.P + 1]);
        if (vol < 0.01) vol = 0.0;
        Q.vol[idx] = vol;
        body_normal(S.bodies[body], nx, ny, x, y);
        cell = (vol == 0.0) ? CELL_SOLID : CELL_FLUID;
    } else {
        cell = (d < 0.0) ? CELL_SOLID : CELL_FLUID;
        body_normal(S.bodies[body], nx, ny, x, y);
    }
    Q.cell[idx] = cell;
    Q.nx[idx] = nx;
    Q.ny[idx] = ny;
    if (cell != CELL_FLUID && (ix == 0 || iy == 0 || ix == Q.w - 1 || iy == Q.h - 1))
        atomicOr(S.flags, FLAG_RING_SOLID);
}
template <typename F>
__global__ void cell_kernel(Scene<F> S) { cell_body(S, blockIdx); }

// ------------------------------------------------------ boundary condition
// setBoundaryCondition (4-solid-boundaries/Fluid.cpp:812-833): the later
// (right / upper) solid cell's write wins, then the domain walls are zeroed.
template <typename F>
__device__ __forceinline__ void bc_body(const Scene<F> &S, const uint3 bid) {
    const int w = S.w, h = S.h, P = S.P;
    const uint8_t *cell = S.q[0].cell, *body = S.q[0].body;
    int fx = bid.x * blockDim.x + threadIdx.x, fy = bid.y * blockDim.y + threadIdx.y;
    const double hx = S.hx;
    if (bid.z == 0) {  // u faces (w+1) x h
        if (fx > w || fy >= h) return;
        F *u = S.q[2].src + fx + (size_t)fy * P;
        if (fx == 0 || fx == w) {
            *u = (F)0.0;
            return;
        }
        size_t c = fx + (size_t)fy * P;
        if (cell[c] == CELL_SOLID)
            *u = (F)body_vel_x(S.bodies[body[c]], fx * hx, (fy + 0.5) * hx);
        else if (cell[c - 1] == CELL_SOLID)
            *u = (F)body_vel_x(S.bodies[body[c - 1]], ((fx - 1) + 1.0) * hx, (fy + 0.5) * hx);
    } else {  // v faces w x (h+1)
        if (fx >= w || fy > h) return;
        F *v = S.q[3].src + fx + (size_t)fy * P;
        if (fy == 0 || fy == h) {
            *v = (F)0.0;
            return;
        }
        size_t c = fx + (size_t)fy * P;
        if (cell[c] == CELL_SOLID)
            *v = (F)body_vel_y(S.bodies[body[c]], (fx + 0.5) * hx, fy * hx);
        else if (cell[c - P] == CELL_SOLID)
            *v = (F)body_vel_y(S.bodies[body[c - P]], (fx + 0.5) * hx, ((fy - 1) + 1.0) * hx);
    }
}
template <typename F>
__global__ void bc_kernel(Scene<F> S) { bc_body(S, blockIdx); }

// ---------------------------------------------------------------- buoyancy
// addBuoyancy (7-variable-density/Fluid.cpp:908-919), gathered per v face.
template <typename F>
__device__ __forceinline__ void buoyancy_body(const Scene<F> &S, double dt, const uint3 bid) {
    int fx = bid.x * blockDim.x + threadIdx.x, fy = bid.y * blockDim.y + threadIdx.y;
    if (fx >= S.w || fy > S.h) return;
    const int P = S.P;
    const double alpha = (S.rho_soot - S.rho_air) / S.rho_air;
    const F *d = S.q[0].src, *t = S.q[1].src;
    F *v = S.q[3].src + fx + (size_t)fy * P;
    double val = (double)*v;
    if (fy > 0) {
        size_t c = fx + (size_t)(fy - 1) * P;
        double b = dt * S.g * (alpha * (double)d[c] - ((double)t[c] - S.t_amb) / S.t_amb);
        val += b * 0.5;
    }
    if (fy < S.h) {
        size_t c = fx + (size_t)fy * P;
        double b = dt * S.g * (alpha * (double)d[c] - ((double)t[c] - S.t_amb) / S.t_amb);
        val += b * 0.5;
    }
    *v = (F)val;
}
template <typename F>
__global__ void buoyancy_kernel(Scene<F> S, double dt) { buoyancy_body(S, dt, blockIdx); }

// ------------------------------------------------------------- assembly
// Cell density of computeDensities (7-variable-density/Fluid.cpp:666-667).
template <typename F>
__device__ __forceinline__ double cell_density(const Scene<F> &S, double alpha, size_t c) {
    double dens = S.rho_air * S.t_amb / (double)S.q[1].src[c] * (1.0 + alpha * (double)S.q[0].src[c]);
    return smax(dens, 0.05 * S.rho_air);
}
// u-face density (x, y), 0 <= x <= w: 0.5*left cell + 0.5*right cell.
template <typename F>
__device__ __forceinline__ double udens_at(const Scene<F> &S, double alpha, int x, int y) {
    double acc = 0.0;
    if (x > 0) acc += 0.5 * cell_density(S, alpha, (x - 1) + (size_t)y * S.P);
    if (x < S.w) acc += 0.5 * cell_density(S, alpha, x + (size_t)y * S.P);
    return acc;
}
// v-face density (x, y), 0 <= y <= h.
template <typename F>
__device__ __forceinline__ double vdens_at(const Scene<F> &S, double alpha, int x, int y) {
    double acc = 0.0;
    if (y > 0) acc += 0.5 * cell_density(S, alpha, x + (size_t)(y - 1) * S.P);
    if (y < S.h) acc += 0.5 * cell_density(S, alpha, x + (size_t)y * S.P);
    return acc;
}

// Pressure-matrix coefficient of the x-face between cells (x-1, y) and (x, y).
template <typename F>
__device__ __forceinline__ double xface_factor(const Scene<F> &S, double scale, double alpha, int x, int y) {
    if (S.variant <= 4) return scale;
    double vol = S.q[2].vol[x + (size_t)y * S.P];
    if (S.variant >= 7) return scale * vol / udens_at(S, alpha, x, y);
    return scale * vol;
}
// y-face between (x, y-1) and (x, y).  Step 7 reads the face density at the
// u-grid flat index x + y*(w+1) of the w-wide v-density array; *present is
// cleared when that index leaves the array.
template <typename F>
__device__ __forceinline__ double yface_factor(const Scene<F> &S, double scale, double alpha, int x, int y,
                                               bool *present) {
    if (S.variant <= 4) return scale;
    double vol = S.q[3].vol[x + (size_t)y * S.P];
    if (S.variant >= 7) {
        long flat = (long)x + (long)y * (S.w + 1);
        if (flat >= (long)S.w * (S.h + 1)) {
            *present = false;
            return 0.0;
        }
        int fx = (int)(flat % S.w), fy = (int)(flat / S.w);
        return scale * vol / vdens_at(S, alpha, fx, fy);
    }
    return scale * vol;
}

// buildRhs + computeDensities + buildPressureMatrix (+ neighbour bits), one
// thread per cell.  References: buildRhs 3-conjugate-gradients/Fluid.cpp:208-217,
// 4-solid-boundaries/Fluid.cpp:614-627, 7-variable-density/Fluid.cpp:624-653;
// buildPressureMatrix 3-conjugate-gradients/Fluid.cpp:222-244,
// 4-solid-boundaries/Fluid.cpp:629-654, 5-curved-boundaries/Fluid.cpp:686-713,
// 7-variable-density/Fluid.cpp:680-707.  The diagonal accumulates its faces
// in the reference's visiting order: lower face, left face, right face, upper
// face.
template <typename F>
__device__ __forceinline__ void assemble_body(const Scene<F> &S, double dt, int what, const uint3 bid) {
    const int w = S.w, h = S.h, P = S.P;
    int x = bid.x * blockDim.x + threadIdx.x, y = bid.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const size_t c = x + (size_t)y * P;
    const size_t k = S.sd.slot(x, y);  // pressure-system arrays are strip-diagonal
    const int var = S.variant;
    const uint8_t *cell = S.q[0].cell;
    const bool plain = var <= 3;
    const bool fl = plain || cell[c] == CELL_FLUID;
    const double alpha = (S.rho_soot - S.rho_air) / S.rho_air;
    const F *U = S.q[2].src, *V = S.q[3].src;

    if (what & ASM_RHS) {
        double scale = 1.0 / S.hx;
        double r;
        if (var <= 4) {
            r = fl ? -scale * ((double)U[c + 1] - (double)U[c] + (double)V[c + P] - (double)V[c]) : 0.0;
        } else if (!fl) {
            r = 0.0;
        } else {
            const double *uv = S.q[2].vol, *vv = S.q[3].vol;
            double uv0 = uv[c], uv1 = uv[c + 1], vv0 = vv[c], vv1 = vv[c + P];
            r = -scale * (uv1 * (double)U[c + 1] - uv0 * (double)U[c] + vv1 * (double)V[c + P] -
                          vv0 * (double)V[c]);
            if (S.nbodies > 0) {
                double vol = S.q[0].vol[c];
                const uint8_t *body = S.q[0].body;
                const double hx = S.hx;
                if (x > 0) r -= (uv0 - vol) * body_vel_x(S.bodies[body[c - 1]], x * hx, (y + 0.5) * hx);
                if (y > 0) r -= (vv0 - vol) * body_vel_y(S.bodies[body[c - P]], (x + 0.5) * hx, y * hx);
                if (x < w - 1)
                    r += (uv1 - vol) * body_vel_x(S.bodies[body[c + 1]], (x + 1.0) * hx, (y + 0.5) * hx);
                if (y < h - 1)
                    r += (vv1 - vol) * body_vel_y(S.bodies[body[c + P]], (x + 0.5) * hx, (y + 1.0) * hx);
            }
        }
        S.r[k] = r;
    }

    if (what & ASM_DENS) {  // face densities for applyPressure (step 7)
        S.udens[c] = (F)udens_at(S, alpha, x, y);
        if (x == w - 1) S.udens[c + 1] = (F)udens_at(S, alpha, w, y);
        S.vdens[c] = (F)vdens_at(S, alpha, x, y);
        if (y == h - 1) S.vdens[c + P] = (F)vdens_at(S, alpha, x, h);
    }

    if (what & ASM_MATRIX) {
        double scale = (var >= 7) ? dt / (S.hx * S.hx) : dt / (S.rho_air * S.hx * S.hx);
        bool fL = x > 0 && (plain || (fl && cell[c - 1] == CELL_FLUID));
        bool fR = x < w - 1 && (plain || (fl && cell[c + 1] == CELL_FLUID));
        bool fD = y > 0 && (plain || (fl && cell[c - P] == CELL_FLUID));
        bool fU = y < h - 1 && (plain || (fl && cell[c + P] == CELL_FLUID));
        double diag = 0.0, ax = 0.0, ay = 0.0;
        if (fD) {
            double f = yface_factor(S, scale, alpha, x, y, &fD);
            if (fD) diag += f;
        }
        if (fL) diag += xface_factor(S, scale, alpha, x, y);
        if (fR) {
            double f = xface_factor(S, scale, alpha, x + 1, y);
            diag += f;
            ax = -f;
        }
        if (fU) {
            double f = yface_factor(S, scale, alpha, x, y + 1, &fU);
            if (fU) {
                diag += f;
                ay = -f;
            }
        }
        S.adiag[k] = (F)diag;
        S.ax[k] = (F)ax;
        S.ay[k] = (F)ay;
        uint8_t nb = (fl ? NB_SELF : 0) | (fL ? NB_LEFT : 0) | (fD ? NB_DOWN : 0) | (fR ? NB_RIGHT : 0) |
                     (fU ? NB_UP : 0) | ((var < 6 || cell[c] == CELL_FLUID) ? NB_RED : 0);
        // The MIC(0) sweeps use the fluid test of each neighbour, independent
        // of whether the face carries a matrix entry.
        if (!plain) {
            nb = (fl ? NB_SELF : 0) | ((var < 6 || fl) ? NB_RED : 0);
            if (x > 0 && cell[c - 1] == CELL_FLUID) nb |= NB_LEFT;
            if (y > 0 && cell[c - P] == CELL_FLUID) nb |= NB_DOWN;
            if (x < w - 1 && cell[c + 1] == CELL_FLUID) nb |= NB_RIGHT;
            if (y < h - 1 && cell[c + P] == CELL_FLUID) nb |= NB_UP;
        }
        S.nb[k] = nb;
    }
}
template <typename F>
__global__ void assemble_kernel(Scene<F> S, double dt, int what) { assemble_body(S, dt, what, blockIdx); }

// r = T, buildHeatDiffusionMatrix (7-variable-density/Fluid.cpp:709-737,
// 1001) and the neighbour bits.
template <typename F>
__device__ __forceinline__ void heat_assemble_body(const Scene<F> &S, double dt, const uint3 bid) {
    const int w = S.w, h = S.h, P = S.P;
    int x = bid.x * blockDim.x + threadIdx.x, y = bid.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const size_t c = x + (size_t)y * P;
    const size_t k = S.sd.slot(x, y);
    const uint8_t *cell = S.q[0].cell;
    const bool fl = cell[c] == CELL_FLUID;
    S.r[k] = (double)S.q[1].src[c];
    double scale = S.diffusion * dt * 1.0 / (S.hx * S.hx);
    bool fL = x > 0 && fl && cell[c - 1] == CELL_FLUID;
    bool fR = x < w - 1 && fl && cell[c + 1] == CELL_FLUID;
    bool fD = y > 0 && fl && cell[c - P] == CELL_FLUID;
    bool fU = y < h - 1 && fl && cell[c + P] == CELL_FLUID;
    double diag = 1.0;
    if (fD) diag += scale;
    if (fL) diag += scale;
    if (fR) diag += scale;
    if (fU) diag += scale;
    S.adiag[k] = (F)diag;
    S.ax[k] = (F)(fR ? -scale : 0.0);
    S.ay[k] = (F)(fU ? -scale : 0.0);
    uint8_t nb = (fl ? NB_SELF : 0) | (fl ? NB_RED : 0);
    if (x > 0 && cell[c - 1] == CELL_FLUID) nb |= NB_LEFT;
    if (y > 0 && cell[c - P] == CELL_FLUID) nb |= NB_DOWN;
    if (x < w - 1 && cell[c + 1] == CELL_FLUID) nb |= NB_RIGHT;
    if (y < h - 1 && cell[c + P] == CELL_FLUID) nb |= NB_UP;
    S.nb[k] = nb;
}
template <typename F>
__global__ void heat_assemble_kernel(Scene<F> S, double dt) { heat_assemble_body(S, dt, blockIdx); }

// ---------------------------------------------------------- applyPressure
// 3-conjugate-gradients/Fluid.cpp:382-398, 4-solid-boundaries/Fluid.cpp:794-809,
// 7-variable-density/Fluid.cpp:891-906, gathered per face: first the
// contribution of the lower/left cell (visited first), then the cell itself.
template <typename F>
__device__ __forceinline__ void apply_pressure_body(const Scene<F> &S, double dt, const uint3 bid) {
    const int w = S.w, h = S.h, P = S.P, var = S.variant;
    int fx = bid.x * blockDim.x + threadIdx.x, fy = bid.y * blockDim.y + threadIdx.y;
    const uint8_t *cell = S.q[0].cell;
    const double scale = (var >= 7) ? dt / S.hx : dt / (S.rho_air * S.hx);
    if (bid.z == 0) {  // u faces
        if (fx > w || fy >= h) return;
        size_t f = fx + (size_t)fy * P;
        F *u = S.q[2].src + f;
        if (var <= 3 && (fx == 0 || fx == w)) {
            *u = (F)0.0;
            return;
        }
        double val = (double)*u;
        if (fx > 0 && (var <= 3 || cell[f - 1] == CELL_FLUID)) {
            double pv = (double)S.p[S.sd.slot(fx - 1, fy)];
            val += (var >= 7) ? scale * pv / (double)S.udens[f] : scale * pv;
        }
        if (fx < w && (var <= 3 || cell[f] == CELL_FLUID)) {
            double pv = (double)S.p[S.sd.slot(fx, fy)];
            val -= (var >= 7) ? scale * pv / (double)S.udens[f] : scale * pv;
        }
        *u = (F)val;
    } else {  // v faces
        if (fx >= w || fy > h) return;
        size_t f = fx + (size_t)fy * P;
        F *v = S.q[3].src + f;
        if (var <= 3 && (fy == 0 || fy == h)) {
            *v = (F)0.0;
            return;
        }
        double val = (double)*v;
        if (fy > 0 && (var <= 3 || cell[f - P] == CELL_FLUID)) {
            double pv = (double)S.p[S.sd.slot(fx, fy - 1)];
            val += (var >= 7) ? scale * pv / (double)S.vdens[f] : scale * pv;
        }
        if (fy < h && (var <= 3 || cell[f] == CELL_FLUID)) {
            double pv = (double)S.p[S.sd.slot(fx, fy)];
            val -= (var >= 7) ? scale * pv / (double)S.vdens[f] : scale * pv;
        }
        *v = (F)val;
    }
}
template <typename F>
__global__ void apply_pressure_kernel(Scene<F> S, double dt) { apply_pressure_body(S, dt, blockIdx); }

// ------------------------------------------------------------ extrapolate
// extrapolate / fillSolidMask / extrapolateNormal (4-solid-boundaries/Fluid.cpp:508-587).
// The reference solves the upwind DAG with a LIFO stack; every interior solid
// cell is computed exactly once, from upstream neighbours that are final, so
// a level-synchronous relaxation over the same DAG gives the same values.
// Pass 1 (grid-wide): mask bits and the list of interior solid cells.
template <typename F>
__device__ __forceinline__ void extrap_mask_body(const Scene<F> &S, unsigned qmask, int *counters, const uint3 bid) {
    int qi = bid.z;
    if (!((qmask >> qi) & 1u)) return;
    Quant<F> Q = S.q[qi];
    int x = bid.x * blockDim.x + threadIdx.x, y = bid.y * blockDim.y + threadIdx.y;
    if (x >= Q.w || y >= Q.h) return;
    const int P = S.P;
    size_t idx = x + (size_t)y * P;
    if (Q.cell[idx] == CELL_FLUID) return;
    Q.ready[idx] = 0;
    if (x < 1 || y < 1 || x >= Q.w - 1 || y >= Q.h - 1) return;
    double nx = Q.nx[idx], ny = Q.ny[idx];
    int m = 0;
    if (nx != 0.0 && Q.cell[idx + sgn(nx)] != CELL_FLUID) m |= 1;
    if (ny != 0.0 && Q.cell[idx + (long)sgn(ny) * P] != CELL_FLUID) m |= 2;
    int slot = atomicAdd(&counters[qi], 1);
    Q.list[slot] = (int)(idx * 4 + m);
}

template <typename F>
__global__ void extrap_mask_kernel(Scene<F> S, unsigned qmask, int *counters) {
    extrap_mask_body(S, qmask, counters, blockIdx);
}

// Pass 2: one CTA per quantity solves the DAG by frontiers.  The first
// frontier holds the listed cells whose upstream neighbours are all fluid
// (mask 0).  A round computes its frontier (every value in it depends only on
// cells that are final); after a barrier, which makes the round's values
// visible to the whole CTA, each computed cell looks at its four neighbours: a
// pending listed cell whose upstream neighbours are now all done joins the
// next frontier, claimed once by an atomic compare-and-swap of its state
// (0 pending, 2 queued, 1 done).  The work is proportional to the solid cells,
// not to cells times the depth of the DAG, and each cell still gets the value
// the reference's stack computes for it.  Cells on an upwind cycle are never
// queued, as the reference never solves them.
template <typename F>
__device__ __forceinline__ bool extrap_claim(uint8_t *ready, long idx) {
    unsigned *w = (unsigned *)((uintptr_t)(ready + idx) & ~(uintptr_t)3);
    const unsigned sh = 8u * (unsigned)((uintptr_t)(ready + idx) & 3);
    unsigned old = *(volatile unsigned *)w;
    for (;;) {
        if ((old >> sh) & 0xffu) return false;
        const unsigned seen = atomicCAS(w, old, old | (2u << sh));
        if (seen == old) return true;
        old = seen;
    }
}

template <typename F>
__device__ __forceinline__ void extrap_solve_body(const Scene<F> &S, unsigned qmask, const int *counters, int qi) {
    if (!((qmask >> qi) & 1u)) return;
    Quant<F> Q = S.q[qi];
    const long P = S.P;
    const size_t cap = (size_t)P * (S.h + 2);
    // the list is read once (first frontier); the frontiers then alternate
    // between the second half and the first half of the list buffer
    const int *lst = Q.list;
    int *cur = Q.list + cap, *nxt = Q.list;
    const int cnt = counters[qi];
    __shared__ int s_n;
    if (threadIdx.x == 0) s_n = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
        const int e = lst[i];
        if ((e & 3) == 0) {
            Q.ready[e >> 2] = 2;
            cur[atomicAdd(&s_n, 1)] = e >> 2;
        }
    }
    __syncthreads();
    int n = s_n;
    __syncthreads();
    while (n > 0) {
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const long idx = cur[i];
            const double nx = Q.nx[idx], ny = Q.ny[idx];
            const long ix = idx + sgn(nx), iy = idx + (long)sgn(ny) * P;
            const double sx = (double)Q.src[ix], sy = (double)Q.src[iy];
            Q.src[idx] = (F)((fabs(nx) * sx + fabs(ny) * sy) / (fabs(nx) + fabs(ny)));
            Q.ready[idx] = 1;
        }
        if (threadIdx.x == 0) s_n = 0;
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const long idx = cur[i];
            const long nbr[4] = {idx - 1, idx + 1, idx - P, idx + P};
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const long j = nbr[k];
                const int x = (int)(j % P), y = (int)(j / P);
                if (x < 1 || y < 1 || x >= Q.w - 1 || y >= Q.h - 1) continue;  // the outer ring is never extrapolated
                if (Q.cell[j] == CELL_FLUID || Q.ready[j] != 0) continue;
                const double nx = Q.nx[j], ny = Q.ny[j];
                const long jx = j + sgn(nx), jy = j + (long)sgn(ny) * P;
                const bool wx = nx != 0.0 && Q.cell[jx] != CELL_FLUID, wy = ny != 0.0 && Q.cell[jy] != CELL_FLUID;
                if ((wx && Q.ready[jx] != 1) || (wy && Q.ready[jy] != 1)) continue;
                if (extrap_claim<F>(Q.ready, j)) nxt[atomicAdd(&s_n, 1)] = (int)j;
            }
        }
        __syncthreads();
        n = s_n;
        int *t = cur;
        cur = nxt;
        nxt = t;
        __syncthreads();
    }
}
template <typename F>
__global__ void __launch_bounds__(1024) extrap_solve_kernel(Scene<F> S, unsigned qmask, const int *counters) {
    extrap_solve_body(S, qmask, counters, blockIdx.x);
}

// Step 8 (FLIP) extrapolation after the particle-to-grid transfer.  Without
// CELL_EMPTY cells it is the DAG above (the outer ring is never extrapolated
// in either form).  With empty cells the result depends on the reference's
// LIFO order - an empty cell averages the neighbours that are fluid when it is
// popped - so one thread per quantity replays the stack exactly; the other
// threads of the CTA build the masks and the initial stack
// (8-flip/Fluid.cpp:478-653).
template <typename F>
__global__ void extrap_mask_guard_kernel(Scene<F> S, unsigned qmask, int *counters, const int *skip) {
    if (skip[blockIdx.z]) return;
    extrap_mask_body(S, qmask, counters, blockIdx);
}
template <typename F>
__global__ void __launch_bounds__(1024)
    extrap_solve_guard_kernel(Scene<F> S, unsigned qmask, const int *counters, const int *skip) {
    if (skip[blockIdx.x]) return;
    extrap_solve_body(S, qmask, counters, blockIdx.x);
}

__global__ void __launch_bounds__(1024) extrap_lifo_kernel(Scene<double> S, unsigned qmask, const int *empties) {
    const int qi = blockIdx.x;
    if (!((qmask >> qi) & 1u) || empties[qi] == 0) return;
    const Quant<double> Q = S.q[qi];
    const int w = Q.w, h = Q.h, P = S.P;
    uint8_t *c = Q.cell, *m = Q.ready;  // `ready` holds the reference's _mask here
    double *src = Q.src;
    const double *nx = Q.nx, *ny = Q.ny;
    int *stack = Q.list;
    const long stack_cap = 2L * P * (S.h + 2);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;

    // fillSolidMask: outer ring 0xFF; solid cells wait for non-fluid upwind
    // neighbours; empty cells with no fluid neighbour wait for any neighbour.
    for (int i = tid; i < w * h; i += blockDim.x) {
        const int x = i % w, y = i / w;
        const long idx = x + (long)y * P;
        uint8_t mv = 0;
        if (x == 0 || y == 0 || x == w - 1 || y == h - 1) {
            mv = 0xFF;
        } else if (c[idx] == CELL_SOLID) {
            const double ax = nx[idx], ay = ny[idx];
            if (ax != 0.0 && c[idx + sgn(ax)] != CELL_FLUID) mv |= 1;
            if (ay != 0.0 && c[idx + (long)sgn(ay) * P] != CELL_FLUID) mv |= 2;
        } else if (c[idx] == CELL_EMPTY) {
            mv = c[idx - 1] != CELL_FLUID && c[idx + 1] != CELL_FLUID && c[idx - P] != CELL_FLUID &&
                 c[idx + P] != CELL_FLUID;
        }
        m[idx] = mv;
    }
    __syncthreads();

    // Initial stack: interior cells in row-major order (ordered compaction).
    __shared__ int s_warp[32];
    __shared__ int s_base, s_total;
    if (tid == 0) s_base = 0;
    __syncthreads();
    const int iw = w - 2, ni = iw > 0 && h > 2 ? iw * (h - 2) : 0;
    for (int base = 0; base < ni; base += blockDim.x) {
        const int i = base + tid;
        long idx = 0;
        bool f = false;
        if (i < ni) {
            idx = 1 + i % iw + (long)(1 + i / iw) * P;
            f = c[idx] != CELL_FLUID && m[idx] == 0;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, f);
        if (lane == 0) s_warp[warp] = __popc(bal);
        __syncthreads();
        if (warp == 0) {
            int v = lane < nwarps ? s_warp[lane] : 0, incl = v;
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            s_warp[lane] = incl - v;
            if (lane == 31) s_total = incl;
        }
        __syncthreads();
        const int total = s_total;
        if (f) stack[s_base + s_warp[warp] + __popc(bal & ((1u << lane) - 1u))] = (int)idx;
        __syncthreads();
        if (tid == 0) s_base += total;
        __syncthreads();
    }

    if (tid == 0) {
        long top = s_base, guard = 0;
        const long limit = 8L * w * h + 64;
        bool bad = false;
        auto push = [&](long v) {
            if (top >= stack_cap) bad = true;
            else stack[top++] = (int)v;
        };
        while (top > 0 && !bad) {
            if (++guard > limit) {
                bad = true;
                break;
            }
            const long idx = stack[--top];
            if (c[idx] == CELL_EMPTY) {  // extrapolateAverage
                double sum = 0.0;
                int k = 0;
                const long nb[4] = {idx - 1, idx + 1, idx - P, idx + P};
                for (int j = 0; j < 4; j++)
                    if (c[nb[j]] == CELL_FLUID) {
                        sum += src[nb[j]];
                        k++;
                    }
                src[idx] = sum / k;
                c[idx] = CELL_FLUID;
            } else {  // extrapolateNormal
                const double ax = nx[idx], ay = ny[idx];
                src[idx] = (fabs(ax) * src[idx + sgn(ax)] + fabs(ay) * src[idx + (long)sgn(ay) * P]) /
                           (fabs(ax) + fabs(ay));
            }
            // freeSolidNeighbour: a solid neighbour whose normal points here
            const long sn[4] = {idx - 1, idx + 1, idx - P, idx + P};
            const bool toward[4] = {nx[idx - 1] > 0.0, nx[idx + 1] < 0.0, ny[idx - P] > 0.0, ny[idx + P] < 0.0};
            for (int j = 0; j < 4; j++) {
                if (!toward[j] || c[sn[j]] != CELL_SOLID) continue;
                m[sn[j]] &= (uint8_t)~(j < 2 ? 1 : 2);
                if (m[sn[j]] == 0) push(sn[j]);
            }
            // freeEmptyNeighbour
            for (int j = 0; j < 4; j++)
                if (c[sn[j]] == CELL_EMPTY && m[sn[j]] == 1) {
                    m[sn[j]] = 0;
                    push(sn[j]);
                }
        }
        if (bad) atomicOr(S.flags, FLAG_FLIP_STACK);
        // extrapolateEmptyBorders: ring cells copy the inward neighbour,
        // corners average two ring cells.
        for (int x = 1; x < w - 1; x++) {
            const long t = x, b = x + (long)(h - 1) * P;
            if (c[t] == CELL_EMPTY) src[t] = src[t + P];
            if (c[b] == CELL_EMPTY) src[b] = src[b - P];
        }
        for (int y = 1; y < h - 1; y++) {
            const long l = (long)y * P, r = (long)y * P + w - 1;
            if (c[l] == CELL_EMPTY) src[l] = src[l + 1];
            if (c[r] == CELL_EMPTY) src[r] = src[r - 1];
        }
        const long tl = 0, tr = w - 1, bl = (long)(h - 1) * P, br = (long)(h - 1) * P + w - 1;
        if (c[tl] == CELL_EMPTY) src[tl] = 0.5 * (src[tl + 1] + src[tl + P]);
        if (c[tr] == CELL_EMPTY) src[tr] = 0.5 * (src[tr - 1] + src[tr + P]);
        if (c[bl] == CELL_EMPTY) src[bl] = 0.5 * (src[bl + 1] + src[bl - P]);
        if (c[br] == CELL_EMPTY) src[br] = 0.5 * (src[br - 1] + src[br - P]);
    }
    __syncthreads();
    for (int i = tid; i < w * h; i += blockDim.x) {
        const long idx = i % w + (long)(i / w) * P;
        if (c[idx] == CELL_EMPTY) c[idx] = CELL_FLUID;
    }
}

// -------------------------------------------------------------- advection

// Catmull-Rom weights of 3-conjugate-gradients/Fluid.cpp:55-69 (computed once
// per fractional offset; the same expressions as the reference).
template <typename F>
struct CerpW {
    F w0, w1, w2, w3;
    __device__ __forceinline__ explicit CerpW(F x) {
        F xsq = x * x;
        F xcu = xsq * x;
        w0 = F(0.0) - F(0.5) * x + F(1.0) * xsq - F(0.5) * xcu;
        w1 = F(1.0) + F(0.0) * x - F(2.5) * xsq + F(1.5) * xcu;
        w2 = F(0.0) + F(0.5) * x + F(2.0) * xsq - F(1.5) * xcu;
        w3 = F(0.0) + F(0.0) * x - F(0.5) * xsq + F(0.5) * xcu;
    }
    __device__ __forceinline__ F apply(F a, F b, F c, F d) const {
        F minV = smin(a, smin(b, smin(c, d)));
        F maxV = smax(a, smax(b, smax(c, d)));
        F t = a * w0 + b * w1 + c * w2 + d * w3;
        return smin(smax(t, minV), maxV);
    }
};

// FluidQuantity::cerp (3-conjugate-gradients/Fluid.cpp:135-152)
template <typename F>
__device__ __forceinline__ F q_cerp(const F *__restrict__ src, int P, int w, int h, F ox, F oy, F x, F y) {
    x = smin(smax(x - ox, F(0.0)), F(w) - F(1.001));
    y = smin(smax(y - oy, F(0.0)), F(h) - F(1.001));
    int ix = (int)x, iy = (int)y;
    x -= F(ix);
    y -= F(iy);
    int x0 = max(ix - 1, 0), x1 = ix, x2 = ix + 1, x3 = min(ix + 2, w - 1);
    int y0 = max(iy - 1, 0), y1 = iy, y2 = iy + 1, y3 = min(iy + 2, h - 1);
    CerpW<F> wx(x), wy(y);
    const F *r0 = src + (size_t)y0 * P, *r1 = src + (size_t)y1 * P;
    const F *r2 = src + (size_t)y2 * P, *r3 = src + (size_t)y3 * P;
    F q0 = wx.apply(__ldg(r0 + x0), __ldg(r0 + x1), __ldg(r0 + x2), __ldg(r0 + x3));
    F q1 = wx.apply(__ldg(r1 + x0), __ldg(r1 + x1), __ldg(r1 + x2), __ldg(r1 + x3));
    F q2 = wx.apply(__ldg(r2 + x0), __ldg(r2 + x1), __ldg(r2 + x2), __ldg(r2 + x3));
    F q3 = wx.apply(__ldg(r3 + x0), __ldg(r3 + x1), __ldg(r3 + x2), __ldg(r3 + x3));
    return wy.apply(q0, q1, q2, q3);
}

// FluidQuantity::advect with rungeKutta3 and backProject
// (3-conjugate-gradients/Fluid.cpp:71-89, 154-165; 4-solid-boundaries/Fluid.cpp:393-427).
// blockIdx.z: 0 = density (and temperature, which shares its grid, cells and
// backtrace), 1 = u, 2 = v.  Every quantity reads the u, v sources and writes
// its own destination, so all of them advect in one launch.
template <typename F>
__device__ __forceinline__ void advect_body(const Scene<F> &S, double dt, const uint3 bid) {
    const int z = bid.z;
    const int qi = z == 0 ? 0 : z + 1;
    const Quant<F> &Q = S.q[qi];
    int ix = bid.x * blockDim.x + threadIdx.x, iy = bid.y * blockDim.y + threadIdx.y;
    if (ix >= Q.w || iy >= Q.h) return;
    const int P = S.P;
    const size_t idx = ix + (size_t)iy * P;
    const bool solid = S.variant >= 4;
    if (solid && Q.cell[idx] != CELL_FLUID) return;
    const Quant<F> &U = S.q[2], &V = S.q[3];
    const F hx = F(S.hx);
    const F uox = F(U.ox), uoy = F(U.oy), vox = F(V.ox), voy = F(V.oy);
    // Positions are FP64 in both forms (the velocity samples and the
    // interpolation run in the storage precision).  u and v faces sit on
    // integer coordinates, where the truncation that selects the
    // back-projection cell is discontinuous: an FP32 position would snap a
    // near-zero displacement onto the face and pick another cell.
    const double fdt = dt;
    double x = ix + Q.ox;
    double y = iy + Q.oy;
    if (S.variant == 1) {  // euler + lerp (1-matrixless/Fluid.cpp:65-73, 124-138)
        F uVel = q_lerp(U.src, P, U.w, U.h, uox, uoy, F(x), F(y)) / hx;
        F vVel = q_lerp(V.src, P, V.w, V.h, vox, voy, F(x), F(y)) / hx;
        x -= (double)uVel * fdt;
        y -= (double)vVel * fdt;
        Q.dst[idx] = q_lerp(Q.src, P, Q.w, Q.h, F(Q.ox), F(Q.oy), F(x), F(y));
        return;
    }
    {
        F firstU = q_lerp(U.src, P, U.w, U.h, uox, uoy, F(x), F(y)) / hx;
        F firstV = q_lerp(V.src, P, V.w, V.h, vox, voy, F(x), F(y)) / hx;
        double midX = x - 0.5 * fdt * (double)firstU;
        double midY = y - 0.5 * fdt * (double)firstV;
        F midU = q_lerp(U.src, P, U.w, U.h, uox, uoy, F(midX), F(midY)) / hx;
        F midV = q_lerp(V.src, P, V.w, V.h, vox, voy, F(midX), F(midY)) / hx;
        double lastX = x - 0.75 * fdt * (double)midU;
        double lastY = y - 0.75 * fdt * (double)midV;
        F lastU = q_lerp(U.src, P, U.w, U.h, uox, uoy, F(lastX), F(lastY));
        F lastV = q_lerp(V.src, P, V.w, V.h, vox, voy, F(lastX), F(lastY));
        x -= fdt * ((2.0 / 9.0) * (double)firstU + (3.0 / 9.0) * (double)midU + (4.0 / 9.0) * (double)lastU);
        y -= fdt * ((2.0 / 9.0) * (double)firstV + (3.0 / 9.0) * (double)midV + (4.0 / 9.0) * (double)lastV);
    }
    if (solid) {
        int rx = min(max((int)(x - Q.ox), 0), Q.w - 1);
        int ry = min(max((int)(y - Q.oy), 0), Q.h - 1);
        size_t r = rx + (size_t)ry * P;
        if (Q.cell[r] != CELL_FLUID) {
            x = (x - Q.ox) * S.hx;
            y = (y - Q.oy) * S.hx;
            body_closest(S.bodies[Q.body[r]], x, y);
            x = x / S.hx + Q.ox;
            y = y / S.hx + Q.oy;
        }
    }
    Q.dst[idx] = q_cerp(Q.src, P, Q.w, Q.h, F(Q.ox), F(Q.oy), F(x), F(y));
    if (z == 0 && S.nq == 4) {
        const Quant<F> &T = S.q[1];
        T.dst[idx] = q_cerp(T.src, P, T.w, T.h, F(T.ox), F(T.oy), F(x), F(y));
    }
}
template <typename F>
__global__ void advect_kernel(Scene<F> S, double dt) { advect_body(S, dt, blockIdx); }

// Strip-diagonal FP64 array -> row-major field (T = p after the heat solve).
template <typename F>
__global__ void sd_to_rows_kernel(SDIdx sd, int P, F *rows, const double *sd_arr) {
    int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= sd.W || y >= sd.H) return;
    rows[x + (size_t)y * P] = (F)sd_arr[sd.slot(x, y)];
}

// ------------------------------------------------------------------ image
// FluidSolver::toImage (3-conjugate-gradients/Fluid.cpp:455-465,
// 4-solid-boundaries/Fluid.cpp:903-916, 5-curved-boundaries/Fluid.cpp:961-972,
// 7-variable-density/Fluid.cpp:1047-1081, 8-flip/Fluid.cpp:1426-1470): 8-bit
// RGBA, row y at y*width; with heat (steps 6-8) the image is 2w wide, heat
// colours left, shade right.
template <typename F>
__global__ void render_kernel(Scene<F> S, unsigned char *rgba, int heat) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    const int w = S.w, h = S.h;
    if (x >= w || y >= h) return;
    const size_t c = x + (size_t)y * S.P;
    const double d = (double)S.q[0].src[c];
    if (S.variant <= 5) {
        int shade = S.variant == 5 ? (int)((1.0 - d) * S.q[0].vol[c] * 255.0) : (int)((1.0 - d) * 255.0);
        shade = shade < 255 ? shade : 255;  // max(min(shade, 255), 0)
        shade = shade < 0 ? 0 : shade;
        if (S.variant == 4 && S.q[0].cell[c] == CELL_SOLID) shade = 0;
        const size_t o = 4 * (x + (size_t)y * w);
        rgba[o] = rgba[o + 1] = rgba[o + 2] = (unsigned char)shade;
        rgba[o + 3] = 0xFF;
        return;
    }
    const double volume = S.q[0].vol[c];
    double shade = (1.0 - d) * volume;
    shade = smin(smax(shade, 0.0), 1.0);
    const size_t oright = heat ? 4 * (x + (size_t)y * w * 2 + w) : 4 * (x + (size_t)y * w);
    rgba[oright] = rgba[oright + 1] = rgba[oright + 2] = (unsigned char)(int)(shade * 255.0);
    rgba[oright + 3] = 0xFF;
    if (S.variant == 8 && S.q[0].cell[c] == CELL_EMPTY) {  // 8-flip/Fluid.cpp:1446-1449
        rgba[oright] = 0xFF;
        rgba[oright + 1] = rgba[oright + 2] = 0;
    }
    if (heat) {
        double t = S.variant == 8 ? fabs((double)S.q[1].src[c] - S.t_amb) / 70.0
                                  : ((double)S.q[1].src[c] - S.t_amb) / 700.0;
        t = smin(smax(t, 0.0), 1.0);
        const double r = 1.0 + volume * (smin(t * 4.0, 1.0) - 1.0);
        const double g = 1.0 + volume * (smin(t * 2.0, 1.0) - 1.0);
        const double b = 1.0 + volume * (smax(smin(t * 4.0 - 3.0, 1.0), 0.0) - 1.0);
        const size_t ol = 4 * (x + (size_t)y * w * 2);
        rgba[ol] = (unsigned char)(int)(r * 255.0);
        rgba[ol + 1] = (unsigned char)(int)(g * 255.0);
        rgba[ol + 2] = (unsigned char)(int)(b * 255.0);
        rgba[ol + 3] = 0xFF;
    }
}

inline dim3 grid2(int nx, int ny, int nz, dim3 b) {
    return dim3((nx + b.x - 1) / b.x, (ny + b.y - 1) / b.y, nz);
}

}  // namespace

// -------------------------------------------------------------- launchers
template <typename F>
void launch_inflow(const Scene<F> &S, int qi, double x0, double y0, double x1, double y1, double val,
                   cudaStream_t st) {
    inflow_kernel<F><<<1, 256, 0, st>>>(S.q[qi], S.P, S.hx, x0, y0, x1, y1, val, S.variant == 1);
}

template <typename F>
void launch_fill_solid(const Scene<F> &S, cudaStream_t st) {
    dim3 b(32, 8);
    if (S.variant >= 5) phi_kernel<F><<<grid2(S.w + 2, S.h + 2, S.nq, b), b, 0, st>>>(S);
    cell_kernel<F><<<grid2(S.w + 1, S.h + 1, S.nq, b), b, 0, st>>>(S);
}

template <typename F>
void launch_bc(const Scene<F> &S, cudaStream_t st) {
    dim3 b(32, 8);
    bc_kernel<F><<<grid2(S.w + 1, S.h + 1, 2, b), b, 0, st>>>(S);
}

template <typename F>
void launch_buoyancy(const Scene<F> &S, double dt, cudaStream_t st) {
    dim3 b(32, 8);
    buoyancy_kernel<F><<<grid2(S.w, S.h + 1, 1, b), b, 0, st>>>(S, dt);
}

template <typename F>
void launch_assemble(const Scene<F> &S, double dt, int what, cudaStream_t st) {
    dim3 b(32, 8);
    assemble_kernel<F><<<grid2(S.w, S.h, 1, b), b, 0, st>>>(S, dt, what);
}

template <typename F>
void launch_heat_assemble(const Scene<F> &S, double dt, cudaStream_t st) {
    dim3 b(32, 8);
    heat_assemble_kernel<F><<<grid2(S.w, S.h, 1, b), b, 0, st>>>(S, dt);
}

template <typename F>
void launch_apply_pressure(const Scene<F> &S, double dt, cudaStream_t st) {
    dim3 b(32, 8);
    apply_pressure_kernel<F><<<grid2(S.w + 1, S.h + 1, 2, b), b, 0, st>>>(S, dt);
}

template <typename F>
void launch_extrapolate(const Scene<F> &S, unsigned qmask, cudaStream_t st) {
    // counters live right after the status word
    int *counters = (int *)(S.flags + 4);
    cudaMemsetAsync(counters, 0, 4 * sizeof(int), st);
    dim3 b(32, 8);
    extrap_mask_kernel<F><<<grid2(S.w + 1, S.h + 1, 4, b), b, 0, st>>>(S, qmask, counters);
    extrap_solve_kernel<F><<<4, 1024, 0, st>>>(S, qmask, counters);
}

void launch_extrapolate_guarded(const Scene<double> &S, unsigned qmask, const int *empty_counts, cudaStream_t st) {
    int *counters = (int *)(S.flags + 4);
    cudaMemsetAsync(counters, 0, 4 * sizeof(int), st);
    dim3 b(32, 8);
    extrap_mask_guard_kernel<double><<<grid2(S.w + 1, S.h + 1, 4, b), b, 0, st>>>(S, qmask, counters, empty_counts);
    extrap_solve_guard_kernel<double><<<4, 1024, 0, st>>>(S, qmask, counters, empty_counts);
    extrap_lifo_kernel<<<4, 1024, 0, st>>>(S, qmask, empty_counts);
}

template <typename F>
void launch_advect(const Scene<F> &S, double dt, cudaStream_t st) {
    dim3 b(32, 8);
    advect_kernel<F><<<grid2(S.w + 1, S.h + 1, 3, b), b, 0, st>>>(S, dt);
}

template <typename F>
void launch_render(const Scene<F> &S, unsigned char *rgba, int heat, cudaStream_t st) {
    dim3 b(32, 8);
    render_kernel<F><<<grid2(S.w, S.h, 1, b), b, 0, st>>>(S, rgba, heat);
}

template <typename F>
void launch_sd_to_rows(const Scene<F> &S, F *rows, const double *sd_arr, cudaStream_t st) {
    dim3 b(32, 8);
    sd_to_rows_kernel<F><<<grid2(S.w, S.h, 1, b), b, 0, st>>>(S.sd, S.P, rows, sd_arr);
}

// ------------------------------------------------------------ batched phases
// One launch runs a phase for every scene of a batch.  A scene covers
// batch_tiles(w, h, tw, th) tiles of tw x th threads (the batch's shape for the
// phase), enough for every grid of the scene (the bodies bound-check their own
// grid and index by blockDim); blockIdx.x enumerates the tiles of all scenes
// through the prefix table tile_start, blockIdx.y is the phase's third grid
// dimension (quantity or face kind).
namespace {

template <typename F>
__device__ __forceinline__ int scene_of_tile(const SceneBatch<F> &B, int t) {
    int lo = 0, hi = B.n;  // largest i with tile_start[i] <= t
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (B.tile_start[mid] <= t) lo = mid;
        else hi = mid;
    }
    return lo;
}

template <typename F, typename Op>
__global__ void __launch_bounds__(256) batch_tiles_kernel(SceneBatch<F> B, Op op) {
    const int i = scene_of_tile(B, blockIdx.x);
    const Scene<F> &S = B.scenes[i];
    const int tx = (S.w + 2 + (int)blockDim.x - 1) / (int)blockDim.x;
    const int local = blockIdx.x - B.tile_start[i];
    op(S, make_uint3(local % tx, local / tx, blockIdx.y));
}

// fillSolidFields returns at once without bodies (4-solid-boundaries/Fluid.cpp:455)
template <typename F> struct PhiOp {
    __device__ void operator()(const Scene<F> &S, uint3 b) const {
        if (S.nbodies > 0) phi_body(S, b);
    }
};
template <typename F> struct CellOp {
    __device__ void operator()(const Scene<F> &S, uint3 b) const {
        if (S.nbodies > 0) cell_body(S, b);
    }
};
template <typename F> struct BcOp {
    __device__ void operator()(const Scene<F> &S, uint3 b) const { bc_body(S, b); }
};
template <typename F> struct BuoyancyOp {
    double dt;
    __device__ void operator()(const Scene<F> &S, uint3 b) const { buoyancy_body(S, dt, b); }
};
template <typename F> struct AssembleOp {
    double dt;
    int what;
    __device__ void operator()(const Scene<F> &S, uint3 b) const { assemble_body(S, dt, what, b); }
};
template <typename F> struct HeatAssembleOp {
    double dt;
    __device__ void operator()(const Scene<F> &S, uint3 b) const { heat_assemble_body(S, dt, b); }
};
template <typename F> struct HeatToRowsOp {  // T = p (7-variable-density/Fluid.cpp:1005)
    __device__ void operator()(const Scene<F> &S, uint3 b) const {
        const int x = b.x * blockDim.x + threadIdx.x, y = b.y * blockDim.y + threadIdx.y;
        if (x >= S.w || y >= S.h) return;
        S.q[1].src[x + (size_t)y * S.P] = (F)S.p[S.sd.slot(x, y)];
    }
};
template <typename F> struct ApplyOp {
    double dt;
    __device__ void operator()(const Scene<F> &S, uint3 b) const { apply_pressure_body(S, dt, b); }
};
template <typename F> struct MaskOp {
    unsigned qmask;
    __device__ void operator()(const Scene<F> &S, uint3 b) const {
        extrap_mask_body(S, qmask, (int *)(S.flags + 4), b);
    }
};
template <typename F> struct AdvectOp {
    double dt;
    __device__ void operator()(const Scene<F> &S, uint3 b) const { advect_body(S, dt, b); }
};

// The inflows of one scene, in call order, by one block.
template <typename F>
__global__ void batch_inflow_kernel(SceneBatch<F> B) {
    const Scene<F> &S = B.scenes[blockIdx.x];
    for (int r = B.inflow_start[blockIdx.x]; r < B.inflow_start[blockIdx.x + 1]; r++) {
        const BatchInflow f = B.inflows[r];
        inflow_body(S.q[f.q], S.P, S.hx, f.x0, f.y0, f.x1, f.y1, f.val);
        __syncthreads();
    }
}

// Extrapolation counters of every scene (Scene::flags[4..8)).
template <typename F>
__global__ void batch_zero_counters_kernel(SceneBatch<F> B) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B.n) return;
    int *c = (int *)(B.scenes[i].flags + 4);
    c[0] = c[1] = c[2] = c[3] = 0;
}

template <typename F>
__global__ void __launch_bounds__(1024) batch_extrap_solve_kernel(SceneBatch<F> B, unsigned qmask) {
    const Scene<F> &S = B.scenes[blockIdx.x];
    extrap_solve_body(S, qmask, (const int *)(S.flags + 4), blockIdx.y);
}

template <typename F, typename Op>
void tiles(const SceneBatch<F> &B, int nz, Op op, cudaStream_t st) {
    if (B.tiles > 0) batch_tiles_kernel<F, Op><<<dim3(B.tiles, nz), dim3(B.tw, B.th), 0, st>>>(B, op);
}

}  // namespace

template <typename F>
void launch_batch_inflow(const SceneBatch<F> &B, cudaStream_t st) {
    if (B.n > 0) batch_inflow_kernel<F><<<B.n, 256, 0, st>>>(B);
}
template <typename F>
void launch_batch_fill_solid(const SceneBatch<F> &B, int variant, int nq, cudaStream_t st) {
    if (variant >= 5) tiles(B, nq, PhiOp<F>{}, st);
    tiles(B, nq, CellOp<F>{}, st);
}
template <typename F>
void launch_batch_bc(const SceneBatch<F> &B, cudaStream_t st) {
    tiles(B, 2, BcOp<F>{}, st);
}
template <typename F>
void launch_batch_buoyancy(const SceneBatch<F> &B, double dt, cudaStream_t st) {
    tiles(B, 1, BuoyancyOp<F>{dt}, st);
}
template <typename F>
void launch_batch_assemble(const SceneBatch<F> &B, double dt, int what, cudaStream_t st) {
    tiles(B, 1, AssembleOp<F>{dt, what}, st);
}
template <typename F>
void launch_batch_heat_assemble(const SceneBatch<F> &B, double dt, cudaStream_t st) {
    tiles(B, 1, HeatAssembleOp<F>{dt}, st);
}
template <typename F>
void launch_batch_heat_to_rows(const SceneBatch<F> &B, cudaStream_t st) {
    tiles(B, 1, HeatToRowsOp<F>{}, st);
}
template <typename F>
void launch_batch_apply_pressure(const SceneBatch<F> &B, double dt, cudaStream_t st) {
    tiles(B, 2, ApplyOp<F>{dt}, st);
}
template <typename F>
void launch_batch_extrapolate(const SceneBatch<F> &B, unsigned qmask, cudaStream_t st) {
    if (B.n <= 0) return;
    batch_zero_counters_kernel<F><<<(B.n + 255) / 256, 256, 0, st>>>(B);
    tiles(B, 4, MaskOp<F>{qmask}, st);
    batch_extrap_solve_kernel<F><<<dim3(B.n, 4), 1024, 0, st>>>(B, qmask);
}
template <typename F>
void launch_batch_advect(const SceneBatch<F> &B, double dt, cudaStream_t st) {
    tiles(B, 3, AdvectOp<F>{dt}, st);
}

#define IFL_BATCH_INST(F)                                                                                  \
    template void launch_batch_inflow<F>(const SceneBatch<F> &, cudaStream_t);                              \
    template void launch_batch_fill_solid<F>(const SceneBatch<F> &, int, int, cudaStream_t);                \
    template void launch_batch_bc<F>(const SceneBatch<F> &, cudaStream_t);                                  \
    template void launch_batch_buoyancy<F>(const SceneBatch<F> &, double, cudaStream_t);                    \
    template void launch_batch_assemble<F>(const SceneBatch<F> &, double, int, cudaStream_t);               \
    template void launch_batch_heat_assemble<F>(const SceneBatch<F> &, double, cudaStream_t);               \
    template void launch_batch_heat_to_rows<F>(const SceneBatch<F> &, cudaStream_t);                        \
    template void launch_batch_apply_pressure<F>(const SceneBatch<F> &, double, cudaStream_t);              \
    template void launch_batch_extrapolate<F>(const SceneBatch<F> &, unsigned, cudaStream_t);               \
    template void launch_batch_advect<F>(const SceneBatch<F> &, double, cudaStream_t);
IFL_BATCH_INST(double)
IFL_BATCH_INST(float)

#define IFL_INST(F)                                                                                        \
    template void launch_inflow<F>(const Scene<F> &, int, double, double, double, double, double,           \
                                   cudaStream_t);                                                          \
    template void launch_fill_solid<F>(const Scene<F> &, cudaStream_t);                                     \
    template void launch_bc<F>(const Scene<F> &, cudaStream_t);                                             \
    template void launch_buoyancy<F>(const Scene<F> &, double, cudaStream_t);                               \
    template void launch_assemble<F>(const Scene<F> &, double, int, cudaStream_t);                          \
    template void launch_heat_assemble<F>(const Scene<F> &, double, cudaStream_t);                          \
    template void launch_apply_pressure<F>(const Scene<F> &, double, cudaStream_t);                         \
    template void launch_extrapolate<F>(const Scene<F> &, unsigned, cudaStream_t);                          \
    template void launch_advect<F>(const Scene<F> &, double, cudaStream_t);                                 \
    template void launch_sd_to_rows<F>(const Scene<F> &, F *, const double *, cudaStream_t);                 \
    template void launch_render<F>(const Scene<F> &, unsigned char *, int, cudaStream_t);
IFL_INST(double)
IFL_INST(float)

}  // namespace ifl
