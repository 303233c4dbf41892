// k_gs.cu - the Gauss-Seidel pressure solve of tutorial steps 1-2 (sm_103a).
//
// project() of 1-matrixless/Fluid.cpp:192-240 (the same in
// 2-better-advection): lexicographic Gauss-Seidel sweeps over the implicit
// five-point stencil with solid walls, p kept from the previous step, until
// the largest change of a sweep is below 1e-5 or 600 sweeps.
//
// A lexicographic sweep is a recurrence on the new values of the left and
// lower cells and the old values of the right and upper cells - the shape of
// the MIC(0) forward substitution - so it runs as a strip wavefront and gives
// the reference's values (and therefore its sweep counts) exactly: one warp
// per 32-row strip, lane l on row 32s + l, step d visits the cell x = d - l of
// every lane (one contiguous strip-diagonal line of p and r).  The left value
// is the lane's own previous result, the lower one comes from lane l - 1 by
// shuffle, or for lane 0 from the strip below once that strip has published
// the diagonal; the right and upper values are still the previous sweep's.
//
// The work per cell is FP64 (GB300 runs FP64 at 1/64 of the FP32 rate), so
// every strip gets an SM of its own: one single-warp CTA per strip in a
// cooperative launch, spread one per SM by a shared-memory reservation.
// Strips hand over through L2 (progress counters, values read with
// ld.global.cg), sweeps end at a grid barrier and the maximum change is the
// maximum of the per-strip maxima, which every CTA forms itself.  Every wait
// is bounded; a timeout sets the status word and an abort word that releases
// every other wait.
#include "ifl_device.cuh"

namespace ifl {

namespace {

constexpr int kGB = 8;  // steps per block of neighbour-strip prefetches

struct GsArgs {
    const double *r;
    double *p;
    SDIdx sd;
    double scale;  // timestep / (density * hx * hx)
    int limit, pinned;
    PcgOut *out;
    unsigned *flags;
    unsigned long long *iter_total;
    unsigned long long *prog;  // S progress counters, then the abort word
    double *smax;              // S per-strip maxima
    unsigned *bar;             // grid barrier: arrivals, generation
};

__device__ __forceinline__ bool gs_aborted(const GsArgs &A) {
    return *(const volatile unsigned long long *)(A.prog + A.sd.S) != 0ull;
}
__device__ __forceinline__ void gs_abort(const GsArgs &A) {
    atomicOr(A.flags, FLAG_TIMEOUT);
    *(volatile unsigned long long *)(A.prog + A.sd.S) = 1ull;
}

// Grid barrier for the single-warp CTAs (lane 0 arrives for the CTA).
__device__ __forceinline__ void gs_grid_sync(const GsArgs &A, unsigned &gen) {
    __syncwarp();
    if ((threadIdx.x & 31) == 0) {
        __threadfence();
        const unsigned n = gridDim.x;
        if (atomicAdd(&A.bar[0], 1u) == n - 1) {
            atomicExch(&A.bar[0], 0u);
            __threadfence();
            atomicExch(&A.bar[1], gen + 1);
        } else {
            long long spins = 0;
            while (ld_volatile(&A.bar[1]) == gen && !gs_aborted(A))
                if (++spins > kSpinLimit) gs_abort(A);
        }
        __threadfence();
    }
    gen++;
    __syncwarp();
}

__global__ void __launch_bounds__(32) gs_kernel(GsArgs A) {
    extern __shared__ unsigned char spread[];  // reserves the SM; never touched
    (void)spread;
    const int lane = threadIdx.x, s = blockIdx.x, S = A.sd.S;
    const int w = A.sd.W, h = A.sd.H, D = A.sd.D;
    const int y = s * 32 + lane;
    const bool row = y < h;
    const int steps = w + 31;  // diagonals of one strip per sweep
    const double scale = A.scale;
    // diag of the reference: scale added once per existing neighbour, in order
    const double d2 = scale + scale, d3 = d2 + scale, d4 = d3 + scale;
    const double *rs = A.r + (size_t)s * D * 32 + lane;
    double *ps = A.p + (size_t)s * D * 32 + lane;
    // lane 31 of strip s-1 at diagonal x + 31, lane 0 of strip s+1 at diagonal x
    const double *below = s > 0 ? A.p + ((size_t)(s - 1) * D + 31) * 32 + 31 : A.p;
    const double *above = s + 1 < S ? A.p + (size_t)(s + 1) * D * 32 : A.p;
    unsigned long long *prog_below = A.prog + (s > 0 ? s - 1 : 0);
    unsigned gen = 0;

    double maxDelta = 0.0;
    int sweeps = 0, status = 2;
    for (int it = 0; it < A.limit; it++) {
        const unsigned long long base = (unsigned long long)it * steps;
        unsigned long long seen = 0;  // last progress read from the strip below
        double lmax = 0.0, prev = 0.0;
        // operands of step d, loaded one step ahead (old values nobody writes
        // before this lane's step d)
        double pold = 0.0, rr = 0.0, right = 0.0, up = 0.0;
        auto load = [&](int d) {
            const int x = d - lane;
            if (row && x >= 0 && x < w) {
                const size_t k = (size_t)d * 32;
                pold = ps[k];
                rr = rs[k];
                right = x < w - 1 ? ps[k + 32] : 0.0;
                if (y < h - 1 && lane < 31) up = ps[k + 33];  // lane 31: the block's prefetch
            }
        };
        load(0);
        for (int d0 = 0; d0 < steps; d0 += kGB) {
            // Values from the neighbouring strips for the kGB steps of this
            // block, fetched once per block by lanes 0..kGB-1 (one L2 round
            // trip instead of one per step): the lower row's new values (the
            // strip below must have finished diagonal x + 31 for each of
            // them) and the upper row's old values (the strip above trails
            // this one, so they are still the previous sweep's).
            double dv = 0.0, uv = 0.0;
            if (s > 0 && d0 < w) {
                if (lane == 0) {
                    const unsigned long long need = base + min(d0 + kGB - 1, w - 1) + 32;
                    if (seen < need) {
                        long long spins = 0;
                        while ((seen = *(const volatile unsigned long long *)prog_below) < need) {
                            if (gs_aborted(A)) break;
                            if (++spins > kSpinLimit) gs_abort(A);
                        }
                    }
                }
                __syncwarp();
                __threadfence();
                if (lane < kGB && d0 + lane < w) dv = __ldcg(below + (size_t)(d0 + lane) * 32);
            }
            if (s + 1 < S && lane < kGB) {
                const int xu = d0 + lane - 31;  // lane 31's column at step d0 + lane
                if (xu >= 0 && xu < w && 32 * s + 31 < h - 1) uv = __ldcg(above + (size_t)xu * 32);
            }
            if (__any_sync(0xffffffffu, gs_aborted(A))) break;
            const int dend = min(d0 + kGB, steps);
            for (int d = d0; d < dend; d++) {
                const int x = d - lane;
                const bool act = row && x >= 0 && x < w;
                double down = __shfl_up_sync(0xffffffffu, prev, 1);
                const double d_blk = __shfl_sync(0xffffffffu, dv, d - d0);
                const double u_blk = __shfl_sync(0xffffffffu, uv, d - d0);
                if (lane == 0) down = d_blk;
                const double c_pold = pold, c_rr = rr, c_right = right;
                const double c_up = lane == 31 ? u_blk : up;
                if (d + 1 < steps) load(d + 1);
                if (act) {
                    const int nb = (x > 0) + (y > 0) + (x < w - 1) + (y < h - 1);
                    const double diag = nb == 4 ? d4 : nb == 3 ? d3 : d2;
                    double off = 0.0;
                    if (x > 0) off -= scale * prev;
                    if (y > 0) off -= scale * down;
                    if (x < w - 1) off -= scale * c_right;
                    if (y < h - 1) off -= scale * c_up;
                    const double np = (c_rr - off) / diag;
                    lmax = smax(lmax, fabs(c_pold - np));
                    ps[(size_t)d * 32] = np;
                    prev = np;
                }
                // publish every 4 diagonals (the strip above trails by 32): a
                // device-scope fence per diagonal would lengthen every step
                if (s + 1 < S && (((d + 1) & 3) == 0 || d + 1 == steps)) {
                    __syncwarp();
                    if (lane == 31) {
                        __threadfence();
                        *(volatile unsigned long long *)(A.prog + s) = base + d + 1;
                    }
                }
            }
        }
        // maximum change: per strip, then over the strips (order-free; NaN
        // changes are ignored as std::max(maxDelta, NaN) ignores them)
        for (int o = 16; o > 0; o >>= 1) lmax = smax(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
        if (lane == 0) *(volatile double *)(A.smax + s) = lmax;
        gs_grid_sync(A, gen);
        double m = 0.0;
        for (int i = lane; i < S; i += 32) m = smax(m, __ldcg(A.smax + i));
        for (int o = 16; o > 0; o >>= 1) m = smax(m, __shfl_xor_sync(0xffffffffu, m, o));
        maxDelta = m;
        sweeps = it + 1;
        const bool aborted = __any_sync(0xffffffffu, gs_aborted(A));
        const bool stop = aborted || (A.pinned >= 0 ? it + 1 >= A.pinned : m < 1e-5);
        // nobody may overwrite smax before every CTA has read it
        gs_grid_sync(A, gen);
        if (stop) {
            status = (A.pinned < 0 && m < 1e-5 && !aborted) ? 0 : 2;
            break;
        }
    }
    if (s == 0 && lane == 0) {
        A.out->iterations = sweeps;
        A.out->status = status;
        A.out->max_error = maxDelta;
        atomicAdd(A.iter_total, (unsigned long long)sweeps);
    }
}

constexpr int kSpreadBytes = 120 * 1024;  // one such CTA per SM

}  // namespace

int gs_max_rows() { return 32 * 4096; }

template <typename F>
cudaError_t launch_gs(const Scene<F> &S, const PcgScratch &X, double dt, int limit, int pinned, cudaStream_t st) {
    const int strips = S.sd.S;
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    int smem = strips <= sms ? kSpreadBytes : 0;
    if (smem) {
        e = cudaFuncSetAttribute(gs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
    }
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gs_kernel, 32, smem);
    if (e != cudaSuccess) return e;
    if ((long)per_sm * sms < strips) return cudaErrorCooperativeLaunchTooLarge;
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
    A.prog = X.halo;       // strips + 1 words (halo holds 2 x S x D)
    A.smax = X.partials;   // strips doubles (partials hold 4 x S x D / 16)
    A.bar = X.barrier;
    e = cudaMemsetAsync(A.prog, 0, sizeof(unsigned long long) * (strips + 1), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(A.bar, 0, 2 * sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    void *args[] = {&A};
    return cudaLaunchCooperativeKernel((const void *)gs_kernel, dim3(strips), dim3(32), args, (size_t)smem, st);
}

template cudaError_t launch_gs<double>(const Scene<double> &, const PcgScratch &, double, int, int, cudaStream_t);
template cudaError_t launch_gs<float>(const Scene<float> &, const PcgScratch &, double, int, int, cudaStream_t);

}  // namespace ifl
