// k_gs.cu - the Gauss-Seidel pressure solve of tutorial steps 1-2 (sm_103a).
//
// project() of 1-matrixless/Fluid.cpp:192-240 (the same in
// 2-better-advection): lexicographic Gauss-Seidel sweeps over the implicit
// five-point stencil with solid walls, p kept from the previous step, until
// the largest change of a sweep is below 1e-5 or 600 sweeps.
//
// A lexicographic sweep is a recurrence on the new values of the left and
// lower cells and the old values of the right and upper cells - the shape of
// the MIC(0) forward substitution - so it runs as the same strip wavefront
// and gives the reference's values (and therefore its sweep counts) exactly:
// one warp per 32-row strip, lane l on row 32s + l, step d visits the cell
// x = d - l of every lane (one contiguous strip-diagonal line of p and r).
// The left value is the lane's own previous result, the lower one comes from
// lane l - 1 by shuffle, or for lane 0 from the strip below once that strip
// has published the diagonal (a progress counter per strip in shared
// memory); the right and upper values are still the previous sweep's.  One
// CTA holds every strip (h <= 1024); sweeps are separated by a CTA barrier
// and the maximum change is reduced over the CTA.
#include "ifl_device.cuh"

namespace ifl {

namespace {

constexpr int kGsMaxStrips = 32;

struct GsArgs {
    const double *r;
    double *p;
    SDIdx sd;
    double scale;  // timestep / (density * hx * hx)
    int limit, pinned;
    PcgOut *out;
    unsigned *flags;
    unsigned long long *iter_total;
};

__global__ void __launch_bounds__(1024) gs_kernel(GsArgs A) {
    const int lane = threadIdx.x & 31, s = threadIdx.x >> 5;
    const int w = A.sd.W, h = A.sd.H, D = A.sd.D;
    const int y = s * 32 + lane;
    const bool row = y < h;
    const int steps = w + 31;  // diagonals of one strip per sweep
    const double scale = A.scale;
    __shared__ volatile long long prog[kGsMaxStrips];
    __shared__ double s_max[kGsMaxStrips];
    __shared__ volatile int s_abort;
    __shared__ int s_stop;
    if (lane == 0) prog[s] = 0;
    if (threadIdx.x == 0) s_abort = 0;
    __syncthreads();

    double maxDelta = 0.0;
    int sweeps = 0, status = 2;
    for (int it = 0; it < A.limit; it++) {
        const long long base = (long long)it * steps;
        double lmax = 0.0, prev = 0.0;
        for (int d = 0; d < steps; d++) {
            const int x = d - lane;
            const bool act = row && x >= 0 && x < w;
            double down = __shfl_up_sync(0xffffffffu, prev, 1);
            if (lane == 0 && s > 0 && x < w) {
                // wait for strip s-1 to finish its diagonal x + 31 of this sweep
                const long long need = base + x + 32;
                long long spins = 0;
                while (prog[s - 1] < need && !s_abort) {
                    if (++spins > kSpinLimit) {
                        atomicOr(A.flags, FLAG_TIMEOUT);
                        s_abort = 1;
                    }
                }
                __threadfence_block();
                down = *(const volatile double *)(A.p + ((size_t)(s - 1) * D + x + 31) * 32 + 31);
            }
            if (__any_sync(0xffffffffu, s_abort)) break;
            if (act) {
                const size_t k = ((size_t)s * D + d) * 32 + lane;
                const double pold = A.p[k], rr = A.r[k];
                const double right = x < w - 1 ? A.p[k + 32] : 0.0;
                double up = 0.0;
                if (y < h - 1)
                    up = lane < 31 ? A.p[k + 33] : A.p[((size_t)(s + 1) * D + d - 31) * 32];
                double diag = 0.0, off = 0.0;
                if (x > 0) {
                    diag += scale;
                    off -= scale * prev;
                }
                if (y > 0) {
                    diag += scale;
                    off -= scale * down;
                }
                if (x < w - 1) {
                    diag += scale;
                    off -= scale * right;
                }
                if (y < h - 1) {
                    diag += scale;
                    off -= scale * up;
                }
                const double np = (rr - off) / diag;
                const double delta = fabs(pold - np);
                lmax = smax(lmax, delta);
                A.p[k] = np;
                prev = np;
            }
            __syncwarp();
            if (lane == 31) {
                __threadfence_block();
                prog[s] = base + d + 1;
            }
        }
        // maximum change over the CTA (max is order-free; NaN changes are
        // ignored as std::max(maxDelta, NaN) ignores them)
        for (int o = 16; o > 0; o >>= 1) lmax = smax(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
        if (lane == 0) s_max[s] = lmax;
        __syncthreads();
        if (threadIdx.x == 0) {
            double m = 0.0;
            for (int i = 0; i < (int)(blockDim.x >> 5); i++) m = smax(m, s_max[i]);
            s_max[0] = m;
            s_stop = s_abort || (A.pinned >= 0 ? it + 1 >= A.pinned : m < 1e-5);
        }
        __syncthreads();
        maxDelta = s_max[0];
        sweeps = it + 1;
        const bool stop = s_stop;
        __syncthreads();
        if (stop) {
            status = (A.pinned < 0 && maxDelta < 1e-5) ? 0 : 2;
            break;
        }
    }
    if (threadIdx.x == 0) {
        A.out->iterations = sweeps;
        A.out->status = status;
        A.out->max_error = maxDelta;
        atomicAdd(A.iter_total, (unsigned long long)sweeps);
    }
}

}  // namespace

int gs_max_rows() { return 32 * kGsMaxStrips; }

template <typename F>
cudaError_t launch_gs(const Scene<F> &S, const PcgScratch &X, double dt, int limit, int pinned, cudaStream_t st) {
    if (S.sd.S > kGsMaxStrips) return cudaErrorInvalidValue;
    GsArgs A;
    A.r = S.r;
    A.p = S.p;
    A.sd = S.sd;
    A.scale = dt / (S.rho_air * S.hx * S.hx);
    A.limit = limit;
    A.pinned = pinned;
    A.out = X.out;
    A.flags = S.flags;
    A.iter_total = X.iter_total;
    gs_kernel<<<1, 32 * S.sd.S, 0, st>>>(A);
    return cudaGetLastError();
}

template cudaError_t launch_gs<double>(const Scene<double> &, const PcgScratch &, double, int, int, cudaStream_t);
template cudaError_t launch_gs<float>(const Scene<float> &, const PcgScratch &, double, int, int, cudaStream_t);

}  // namespace ifl
