// k_pcg.cu - MIC(0)-preconditioned conjugate gradients as one persistent
// cooperative kernel per solve (sm_103a).
//
// Reference: FluidSolver::project (3-conjugate-gradients/Fluid.cpp:349-380),
// buildPreconditioner (:247-272), applyPreconditioner (:275-304),
// matrixVectorProduct (:315-332), dotProduct/scaledAdd/infinityNorm (:307-346);
// masked forms in 4-solid-boundaries/Fluid.cpp:656-721 and
// 6-heat/Fluid.cpp:781-826.
//
// Work decomposition
//  * Elementwise phases (fused s-update + matvec + dot; AXPYs + max-norm):
//    grid-stride over cells, per-block partial sums in FP64, a fixed-order
//    cross-block reduction that every block performs identically, so all
//    blocks take the same branch and the result is run-to-run deterministic.
//  * MIC(0) factor and both triangular solves: anti-diagonal wavefronts.  A
//    warp owns a 32-row strip; lane y handles row y and lags lane y-1 by one
//    step, receiving the lower neighbour through a register shuffle.  The
//    strip below publishes its progress (columns completed in its top row)
//    through a release flag that the next strip's lane 0 waits on.  Every cell
//    performs exactly the reference's arithmetic in a dependency-respecting
//    order, so the factor and the solves are bit-identical to the sequential
//    loops.
//  * Phases are separated by a grid barrier of this file (bounded waits).
// Every wait is bounded: on timeout the status word gets FLAG_TIMEOUT, waits
// stop waiting, the kernel runs to its end and the host reports an error.
#include "ifl_device.cuh"

namespace ifl {

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr long long kWaitLimit = 1ll << 22;  // ~1 s of polling
constexpr double kTau = 0.97, kSigma = 0.25, kTol = 1e-5;

template <typename F>
struct PcgArgs {
    int w, h, P, nstrips;
    const F *adiag, *ax, *ay;
    double *pc;
    F *pcf, *lx, *ly;
    const uint8_t *nb;
    F *r, *p, *z, *sa, *sb, *as;
    double *partials;
    unsigned *barrier, *progress, *flags;
    PcgOut *out;
    int mode, limit, pinned;
};

__device__ __forceinline__ bool timed_out(const unsigned *flags) { return ld_volatile(flags) & FLAG_TIMEOUT; }

// Grid barrier: arrival counter + generation word.
__device__ void grid_barrier(unsigned *bar, unsigned *flags) {
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned g = ld_volatile(bar + 1);
        __threadfence();
        unsigned arrived = atomicAdd(bar, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            long long n = 0;
            while (ld_volatile(bar + 1) == g) {
                if (++n > kWaitLimit || timed_out(flags)) {
                    atomicOr(flags, FLAG_TIMEOUT);
                    break;
                }
            }
        }
        __threadfence();
    }
    __syncthreads();
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) v = smax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

// Block partial -> partials[slot*G + block] (fixed order).
__device__ void block_store(double v, bool is_max, double *partials, int slot, double *sm) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = is_max ? warp_max(v) : warp_sum(v);
    if (lane == 0) sm[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double acc = sm[0];
        for (int i = 1; i < kWarps; i++) acc = is_max ? smax(acc, sm[i]) : acc + sm[i];
        partials[slot * gridDim.x + blockIdx.x] = acc;
    }
    __syncthreads();
}

// Every block reduces partials[slot][0..G) in the same fixed order.
__device__ double grid_reduce(const double *partials, int slot, bool is_max, double *sm) {
    const int lane = threadIdx.x & 31;
    if (threadIdx.x < 32) {
        double acc = 0.0;
        const volatile double *p = partials + slot * gridDim.x;
        for (int i = lane; i < (int)gridDim.x; i += 32) acc = is_max ? smax(acc, (double)p[i]) : acc + p[i];
        acc = is_max ? warp_max(acc) : warp_sum(acc);
        if (lane == 0) sm[kWarps] = acc;
    }
    __syncthreads();
    double r = sm[kWarps];
    __syncthreads();
    return r;
}

template <typename T> __device__ __forceinline__ T shfl_up1(T v) { return __shfl_up_sync(0xffffffffu, v, 1); }

template <typename T> __device__ __forceinline__ T ld_cg(const T *p) { return __ldcg(p); }

// Products for the dot: exact FP64 products of the stored values.
__device__ __forceinline__ double dacc(double acc, double a, double b) { return acc + a * b; }
__device__ __forceinline__ double dacc(double acc, float a, float b) { return fma((double)a, (double)b, acc); }

// One 32-row strip of a wavefront sweep.
// KIND 0: MIC(0) factor (FP64), KIND 1: forward solve L q = r,
// KIND 2: backward solve L^T z = q (+ partial dot(z, r)).
template <int KIND, typename F>
__device__ void sweep_strip(const PcgArgs<F> &A, int s, unsigned sid, double &dot) {
    using V = typename std::conditional<KIND == 0, double, F>::type;
    const int lane = threadIdx.x & 31;
    const int w = A.w, h = A.h, P = A.P;
    const int ys = s * 32 + lane;
    const bool rowok = ys < h;
    const int y = (KIND == 2) ? h - 1 - ys : ys;
    const unsigned tag = sid << 16;
    const V *out_below;
    if constexpr (KIND == 0) out_below = A.pc;
    else out_below = A.z;
    V prev = V(0);
    unsigned seen = 0;
    const bool publish = (lane == 31) && (s + 1 < A.nstrips);
    for (int t = 0; t < w + 31; ++t) {
        const int xs = t - lane;
        V below = shfl_up1(prev);
        const bool active = rowok && xs >= 0 && xs < w;
        const int x = (KIND == 2) ? w - 1 - xs : xs;
        if (lane == 0 && s > 0 && active) {
            if (seen <= (unsigned)xs) {
                long long n = 0;
                unsigned v;
                for (;;) {
                    v = ld_volatile(A.progress + s - 1);
                    if (v >= tag + (unsigned)xs + 1u) break;
                    if (++n > kWaitLimit || timed_out(A.flags)) {
                        atomicOr(A.flags, FLAG_TIMEOUT);
                        v = tag + (unsigned)w;
                        break;
                    }
                }
                __threadfence();
                seen = v - tag;
            }
            const int yb = (KIND == 2) ? y + 1 : y - 1;
            below = ld_cg(out_below + x + (size_t)yb * P);
        }
        V val = prev;
        if (active) {
            const size_t c = x + (size_t)y * P;
            const uint8_t b = A.nb[c];
            if (b & NB_SELF) {
                if constexpr (KIND == 0) {
                    // buildPreconditioner (3-conjugate-gradients/Fluid.cpp:253-269)
                    const double diag = (double)A.adiag[c];
                    double e = diag;
                    if (b & NB_LEFT) {
                        double px = (double)A.ax[c - 1] * prev;
                        double py = (double)A.ay[c - 1] * prev;
                        e = e - (px * px + kTau * px * py);
                    }
                    if (b & NB_DOWN) {
                        double px = (double)A.ax[c - P] * below;
                        double py = (double)A.ay[c - P] * below;
                        e = e - (py * py + kTau * px * py);
                    }
                    if (e < kSigma * diag) e = diag;
                    double pc = 1.0 / sqrt(e);
                    A.pc[c] = pc;
                    A.pcf[c] = (F)pc;
                    A.lx[c] = (F)((double)A.ax[c] * pc);
                    A.ly[c] = (F)((double)A.ay[c] * pc);
                    val = pc;
                } else if constexpr (KIND == 1) {
                    // forward substitution (3-conjugate-gradients/Fluid.cpp:276-287)
                    F tt = A.r[c];
                    if (b & NB_LEFT) tt = tt - A.lx[c - 1] * prev;
                    if (b & NB_DOWN) tt = tt - A.ly[c - P] * below;
                    val = tt * A.pcf[c];
                    A.z[c] = val;
                } else {
                    // backward substitution (3-conjugate-gradients/Fluid.cpp:289-303)
                    F tt = A.z[c];
                    if (b & NB_RIGHT) tt = tt - A.lx[c] * prev;
                    if (b & NB_UP) tt = tt - A.ly[c] * below;
                    val = tt * A.pcf[c];
                    A.z[c] = val;
                    if (b & NB_RED) dot = dacc(dot, val, A.r[c]);
                }
            }
        }
        prev = val;
        if (publish && active && ((((xs + 1) & 15) == 0) || xs == w - 1)) {
            __threadfence();
            st_volatile(A.progress + s, tag + (unsigned)xs + 1u);
        }
    }
}

template <int KIND, typename F>
__device__ double sweep(const PcgArgs<F> &A, unsigned sid) {
    const int warp = threadIdx.x >> 5;
    const int total = gridDim.x * kWarps;
    double dot = 0.0;
    // strip s -> block s % G, warp s / G: consecutive strips on different SMs
    for (int s = blockIdx.x + warp * gridDim.x; s < A.nstrips; s += total) sweep_strip<KIND, F>(A, s, sid, dot);
    return dot;
}

template <typename F>
__global__ void __launch_bounds__(kThreads) pcg_kernel(PcgArgs<F> A) {
    __shared__ double sm[kWarps + 1];
    const int w = A.w, h = A.h, P = A.P;
    const int n = w * h;
    const int gtid = blockIdx.x * kThreads + threadIdx.x;
    const int gstride = gridDim.x * kThreads;
    unsigned sid = 1;

    if (A.mode & PCG_FACTOR) {
        sweep<0, F>(A, sid++);
        grid_barrier(A.barrier, A.flags);
    }
    if (!(A.mode & PCG_SOLVE)) return;

    // p = 0; maxError = |r|_inf   (3-conjugate-gradients/Fluid.cpp:350, 354)
    double mx = 0.0;
    for (int i = gtid; i < n; i += gstride) {
        int y = i / w, x = i - y * w;
        size_t c = x + (size_t)y * P;
        A.p[c] = F(0);
        if (A.nb[c] & NB_RED) mx = smax(mx, (double)fabs(A.r[c]));
    }
    block_store(mx, true, A.partials, 0, sm);
    // z = M^-1 r  (:351)
    sweep<1, F>(A, sid++);
    grid_barrier(A.barrier, A.flags);
    double d = sweep<2, F>(A, sid++);
    block_store(d, false, A.partials, 2, sm);
    grid_barrier(A.barrier, A.flags);

    double maxError = grid_reduce(A.partials, 0, true, sm);
    double sigma = grid_reduce(A.partials, 2, false, sm);
    int iterations = 0, status;
    if (A.pinned >= 0 ? A.pinned == 0 : maxError < kTol) {
        status = 1;
    } else {
        status = 2;
        double beta = 0.0;
        F *s_old = A.sa, *s_new = A.sb;
        for (int iter = 0; iter < A.limit; iter++) {
            if (timed_out(A.flags)) break;
            // s = z + beta*s (first iteration: s = z), then z' = A s and z'.s
            double dacc_ = 0.0;
            const F fbeta = (F)beta;
            for (int i = gtid; i < n; i += gstride) {
                int y = i / w, x = i - y * w;
                size_t c = x + (size_t)y * P;
                auto snew = [&](size_t k) -> F {
                    if (iter == 0) return A.z[k];
                    return (A.nb[k] & NB_RED) ? F(A.z[k] + s_old[k] * fbeta) : s_old[k];
                };
                F sc = snew(c);
                F t = A.adiag[c] * sc;
                if (x > 0) t += A.ax[c - 1] * snew(c - 1);
                if (y > 0) t += A.ay[c - P] * snew(c - P);
                if (x < w - 1) t += A.ax[c] * snew(c + 1);
                if (y < h - 1) t += A.ay[c] * snew(c + P);
                s_new[c] = sc;
                A.as[c] = t;
                if (A.nb[c] & NB_RED) dacc_ = dacc(dacc_, t, sc);
            }
            block_store(dacc_, false, A.partials, 1, sm);
            grid_barrier(A.barrier, A.flags);
            const double alpha = sigma / grid_reduce(A.partials, 1, false, sm);
            // p += alpha s; r -= alpha z'; maxError = |r|_inf  (:363-366)
            const F falpha = (F)alpha, fnalpha = (F)(-alpha);
            mx = 0.0;
            for (int i = gtid; i < n; i += gstride) {
                int y = i / w, x = i - y * w;
                size_t c = x + (size_t)y * P;
                if (A.nb[c] & NB_RED) {
                    A.p[c] = A.p[c] + s_new[c] * falpha;
                    F rn = A.r[c] + A.as[c] * fnalpha;
                    A.r[c] = rn;
                    mx = smax(mx, (double)fabs(rn));
                }
            }
            block_store(mx, true, A.partials, 0, sm);
            grid_barrier(A.barrier, A.flags);
            maxError = grid_reduce(A.partials, 0, true, sm);
            iterations = iter + 1;
            if (A.pinned >= 0 ? iterations >= A.pinned : maxError < kTol) {
                status = 0;
                break;
            }
            // z = M^-1 r; sigmaNew = z.r  (:372-376)
            sweep<1, F>(A, sid++);
            grid_barrier(A.barrier, A.flags);
            d = sweep<2, F>(A, sid++);
            block_store(d, false, A.partials, 2, sm);
            grid_barrier(A.barrier, A.flags);
            const double sigmaNew = grid_reduce(A.partials, 2, false, sm);
            beta = sigmaNew / sigma;
            sigma = sigmaNew;
            F *tmp = s_old;
            s_old = s_new;
            s_new = tmp;
        }
        if (status == 2) iterations = A.limit;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        A.out->iterations = iterations;
        A.out->status = status;
        A.out->max_error = maxError;
    }
}

template <typename F>
int max_coresident() {
    static int cached = -1;
    if (cached < 0) {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, pcg_kernel<F>, kThreads, 0);
        cached = sms * (per > 2 ? 2 : per);
    }
    return cached;
}

}  // namespace

template <typename F>
int pcg_max_blocks() {
    return max_coresident<F>();
}

template <typename F>
cudaError_t launch_pcg(const Scene<F> &S, const PcgScratch &X, const PcgConfig &cfg, cudaStream_t st,
                       int *blocks_used) {
    PcgArgs<F> A;
    A.w = S.w;
    A.h = S.h;
    A.P = S.P;
    A.nstrips = (S.h + 31) / 32;
    A.adiag = S.adiag;
    A.ax = S.ax;
    A.ay = S.ay;
    A.pc = S.pc;
    A.pcf = S.pcf;
    A.lx = S.lx;
    A.ly = S.ly;
    A.nb = S.nb;
    A.r = S.r;
    A.p = S.p;
    A.z = S.z;
    A.sa = S.sa;
    A.sb = S.sb;
    A.as = S.as;
    A.partials = X.partials;
    A.barrier = X.barrier;
    A.progress = X.progress;
    A.flags = S.flags;
    A.out = X.out + (cfg.heat ? 1 : 0);
    A.mode = cfg.mode;
    A.limit = cfg.limit;
    A.pinned = cfg.pinned;
    int maxb = max_coresident<F>();
    if (maxb > X.max_blocks) maxb = X.max_blocks;
    int want = (S.w * S.h + kThreads * 4 - 1) / (kThreads * 4);
    if (want < A.nstrips) want = A.nstrips;
    int G = want < maxb ? want : maxb;
    if (G < 1) G = 1;
    if (blocks_used) *blocks_used = G;
    cudaMemsetAsync(X.barrier, 0, 2 * sizeof(unsigned), st);
    cudaMemsetAsync(X.progress, 0, (size_t)A.nstrips * sizeof(unsigned), st);
    void *args[] = {&A};
    return cudaLaunchCooperativeKernel((const void *)pcg_kernel<F>, dim3(G), dim3(kThreads), args, 0, st);
}

template cudaError_t launch_pcg<double>(const Scene<double> &, const PcgScratch &, const PcgConfig &,
                                        cudaStream_t, int *);
template cudaError_t launch_pcg<float>(const Scene<float> &, const PcgScratch &, const PcgConfig &,
                                       cudaStream_t, int *);
template int pcg_max_blocks<double>();
template int pcg_max_blocks<float>();

}  // namespace ifl
