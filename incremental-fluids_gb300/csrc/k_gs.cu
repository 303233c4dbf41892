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
// the diagonal; the right and upper values are the previous sweep's.
//
// Consecutive sweeps overlap: sweep k reads the previous values from buffer
// k & 1 and writes buffer (k + 1) & 1 (p and the scene's otherwise unused A*s
// array), so a strip starts sweep k + 1 as soon as the strip above it has
// passed the columns it needs in sweep k, instead of waiting for the whole
// sweep.  The convergence test of sweep k is taken at the start of sweep
// k + 2 (every strip has then finished sweep k), so at most one sweep runs
// ahead of the test; when sweep k converged that extra sweep is discarded
// (its output went to the other buffer).  The sweep count and every value are
// those of the sequential loop.
//
// The work per cell is FP64 (GB300 runs FP64 at 1/64 of the FP32 rate), so
// every strip gets an SM of its own: one single-warp CTA per strip in a
// cooperative launch, spread one per SM by a shared-memory reservation.
// Strips hand over through L2 (progress counters, values read with
// ld.global.cg); the maximum change of a sweep is the maximum of the per-strip
// maxima, which every CTA forms itself.  Every wait is bounded; a timeout sets
// the status word and an abort word that releases every other wait.
#include "ifl_device.cuh"

namespace ifl {

namespace {

constexpr int kGB = 8;          // steps per block of neighbour-strip prefetches
constexpr int kMaxSlots = 4;    // per-sweep maxima kept (sweep k in slot k % 4)
constexpr double kGsTol = 1e-5;

struct GsArgs {
    const double *r;
    double *buf[2];  // p (sweep k reads buf[k & 1], writes buf[(k + 1) & 1])
    SDIdx sd;
    double scale;  // timestep / (density * hx * hx)
    int limit, pinned;
    long long spin_limit;  // polls of one progress-counter wait before the solve gives up
    PcgOut *out;
    unsigned *flags;
    unsigned long long *iter_total;
    unsigned long long *prog;  // S progress counters (steps done over all sweeps), then the abort word
    double *smax;              // kMaxSlots x S per-strip maxima
};

__device__ __forceinline__ bool gs_aborted(const GsArgs &A) {
    return *(const volatile unsigned long long *)(A.prog + A.sd.S) != 0ull;
}
__device__ __forceinline__ void gs_abort(const GsArgs &A) {
    atomicOr(A.flags, FLAG_TIMEOUT);
    *(volatile unsigned long long *)(A.prog + A.sd.S) = 1ull;
}
// Lane-0 wait until strip i has done `need` steps in total.
__device__ __forceinline__ void gs_wait(const GsArgs &A, int i, unsigned long long need, unsigned long long &seen) {
    if (seen >= need) return;
    long long spins = 0;
    while ((seen = *(const volatile unsigned long long *)(A.prog + i)) < need) {
        if (gs_aborted(A)) return;
        if (++spins > A.spin_limit) gs_abort(A);
    }
}
// Whole warp: every strip has done `need` steps (finished a sweep).
__device__ __forceinline__ void gs_wait_all(const GsArgs &A, unsigned long long need) {
    const int lane = threadIdx.x & 31;
    for (int i = lane; i < A.sd.S; i += 32) {
        unsigned long long seen = 0;
        gs_wait(A, i, need, seen);
    }
    __syncwarp();
    __threadfence();
}
// Maximum change of sweep k over all strips (whole warp; order-free, and NaN
// changes are ignored as std::max(maxDelta, NaN) ignores them).
__device__ __forceinline__ double gs_sweep_max(const GsArgs &A, int k) {
    const int lane = threadIdx.x & 31;
    const double *slot = A.smax + (size_t)(k % kMaxSlots) * A.sd.S;
    double m = 0.0;
    for (int i = lane; i < A.sd.S; i += 32) m = smax(m, __ldcg(slot + i));
    for (int o = 16; o > 0; o >>= 1) m = smax(m, __shfl_xor_sync(0xffffffffu, m, o));
    return m;
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
    const size_t own = (size_t)s * D * 32 + lane;
    // lane 31 of strip s-1 at diagonal x + 31, lane 0 of strip s+1 at diagonal x
    const size_t below = s > 0 ? ((size_t)(s - 1) * D + 31) * 32 + 31 : 0;
    const size_t above = s + 1 < S ? (size_t)(s + 1) * D * 32 : 0;
    const bool top_row = 32 * s + 31 < h - 1;  // lane 31 has an upper neighbour
    const int nsweeps = A.pinned >= 0 ? min(A.limit, A.pinned) : A.limit;

    int final_sweeps = -1, status = 2;
    for (int it = 0; it < nsweeps; it++) {
        if (A.pinned < 0 && it >= 2) {  // the convergence test of sweep it - 2
            gs_wait_all(A, (unsigned long long)(it - 1) * steps);
            if (gs_sweep_max(A, it - 2) < kGsTol) {
                final_sweeps = it - 1;
                status = 0;
                break;
            }
        }
        if (__any_sync(0xffffffffu, gs_aborted(A))) break;
        const double *oldb = A.buf[it & 1];
        double *newb = A.buf[(it + 1) & 1];
        const double *ps_old = oldb + own;
        double *ps_new = newb + own;
        const unsigned long long base = (unsigned long long)it * steps;
        unsigned long long seen_below = 0, seen_above = 0;
        double lmax = 0.0, prev = 0.0;
        // operands of step d, loaded one step ahead (previous-sweep values of
        // this strip's own cells)
        double pold = 0.0, rr = 0.0, right = 0.0, up = 0.0;
        auto load = [&](int d) {
            const int x = d - lane;
            if (row && x >= 0 && x < w) {
                const size_t k = (size_t)d * 32;
                pold = ps_old[k];
                rr = rs[k];
                right = x < w - 1 ? ps_old[k + 32] : 0.0;
                if (y < h - 1 && lane < 31) up = ps_old[k + 33];  // lane 31: the block's prefetch
            }
        };
        load(0);
        for (int d0 = 0; d0 < steps; d0 += kGB) {
            // Neighbour-strip values for the kGB steps of this block, fetched
            // once per block by lanes 0..kGB-1: the lower row's values of this
            // sweep (the strip below must have finished diagonal x + 31) and
            // the upper row's values of the previous sweep (the strip above
            // must have passed column x in that sweep; in sweep 0 they are the
            // initial p, which no sweep 0 writes).
            double dv = 0.0, uv = 0.0;
            if (lane == 0) {
                if (s > 0 && d0 < w) gs_wait(A, s - 1, base + min(d0 + kGB - 1, w - 1) + 32, seen_below);
                const int xu_hi = min(d0 + kGB - 1 - 31, w - 1);
                if (s + 1 < S && top_row && it > 0 && xu_hi >= 0)
                    gs_wait(A, s + 1, base - steps + xu_hi + 1, seen_above);
            }
            __syncwarp();
            __threadfence();
            if (s > 0 && lane < kGB && d0 + lane < w) dv = __ldcg(newb + below + (size_t)(d0 + lane) * 32);
            if (s + 1 < S && top_row && lane < kGB) {
                const int xu = d0 + lane - 31;  // lane 31's column at step d0 + lane
                if (xu >= 0 && xu < w) uv = __ldcg(oldb + above + (size_t)xu * 32);
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
                    ps_new[(size_t)d * 32] = np;
                    prev = np;
                }
                const bool last = d + 1 == steps;
                if (last) {  // this strip's maximum change, before the sweep's last publication
                    double m = lmax;
                    for (int o = 16; o > 0; o >>= 1) m = smax(m, __shfl_xor_sync(0xffffffffu, m, o));
                    if (lane == 0) *(volatile double *)(A.smax + (size_t)(it % kMaxSlots) * S + s) = m;
                }
                // publish every 4 diagonals and at the end of the sweep: a
                // device-scope fence per diagonal would lengthen every step
                // (every lane's stores fenced, since the strips above and below
                // read this strip's last and first rows)
                if (((d + 1) & 3) == 0 || last) {
                    __threadfence();
                    __syncwarp();
                    if (lane == 0) *(volatile unsigned long long *)(A.prog + s) = base + d + 1;
                }
            }
        }
    }
    const bool aborted = __any_sync(0xffffffffu, gs_aborted(A));
    double maxDelta = 0.0;
    if (final_sweeps < 0) {  // no early stop: the tests of the last sweeps are still open
        final_sweeps = nsweeps;
        if (nsweeps > 0 && !aborted) {
            gs_wait_all(A, (unsigned long long)nsweeps * steps);
            maxDelta = gs_sweep_max(A, nsweeps - 1);
            status = 2;
            if (A.pinned < 0) {
                if (nsweeps >= 2 && gs_sweep_max(A, nsweeps - 2) < kGsTol) {
                    final_sweeps = nsweeps - 1;
                    maxDelta = gs_sweep_max(A, nsweeps - 2);
                    status = 0;
                } else if (maxDelta < kGsTol) {
                    status = 0;
                }
            }
        }
    } else {
        maxDelta = gs_sweep_max(A, final_sweeps - 1);
    }
    if (aborted) status = 2;
    // the result is in buf[final & 1]; move it to p (this strip's own cells,
    // after this strip's last sweep, so nothing of this strip writes them later)
    if ((final_sweeps & 1) && !aborted) {
        for (int d = 0; d < steps; d++) {
            const int x = d - lane;
            if (row && x >= 0 && x < w) A.buf[0][own + (size_t)d * 32] = A.buf[1][own + (size_t)d * 32];
        }
    }
    if (s == 0 && lane == 0) {
        A.out->iterations = final_sweeps;
        A.out->status = status;
        A.out->max_error = maxDelta;
        atomicAdd(A.iter_total, (unsigned long long)final_sweeps);
    }
}

constexpr int kSpreadBytes = 120 * 1024;  // one such CTA per SM

}  // namespace

int gs_max_rows() { return 32 * 4096; }

template <typename F>
cudaError_t launch_gs(const Scene<F> &S, const PcgScratch &X, double dt, int limit, int pinned, cudaStream_t st,
                      long long wait_limit) {
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
    A.buf[0] = S.p;
    A.buf[1] = S.as;  // A*s is not used by the Gauss-Seidel steps
    A.sd = S.sd;
    A.scale = dt / (S.rho_air * S.hx * S.hx);
    A.limit = limit;
    A.pinned = pinned;
    A.spin_limit = wait_limit > 0 ? wait_limit : kSpinLimit;
    A.out = X.out;
    A.flags = S.flags;
    A.iter_total = X.iter_total;
    A.prog = X.halo;      // strips + 1 words (halo holds 2 x S x D)
    A.smax = X.partials;  // kMaxSlots x strips doubles (partials hold 4 x S x D / 16)
    e = cudaMemsetAsync(A.prog, 0, sizeof(unsigned long long) * (strips + 1), st);
    if (e != cudaSuccess) return e;
    void *args[] = {&A};
    return cudaLaunchCooperativeKernel((const void *)gs_kernel, dim3(strips), dim3(32), args, (size_t)smem, st);
}

template cudaError_t launch_gs<double>(const Scene<double> &, const PcgScratch &, double, int, int, cudaStream_t,
                                       long long);
template cudaError_t launch_gs<float>(const Scene<float> &, const PcgScratch &, double, int, int, cudaStream_t,
                                      long long);

}  // namespace ifl
