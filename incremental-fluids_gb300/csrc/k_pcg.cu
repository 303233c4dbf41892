// k_pcg.cu - MIC(0)-preconditioned conjugate gradients as one persistent
// cooperative kernel per solve (sm_103a).
//
// Reference: FluidSolver::project (3-conjugate-gradients/Fluid.cpp:349-380),
// buildPreconditioner (:247-272), applyPreconditioner (:275-304),
// matrixVectorProduct (:315-332), dotProduct/scaledAdd/infinityNorm (:307-346);
// masked forms in 4-solid-boundaries/Fluid.cpp:656-721 and
// 6-heat/Fluid.cpp:781-826.
//
// Data: every array of the pressure system is in the strip-diagonal layout
// (SDIdx): a 32-row strip stores its cells diagonal by diagonal, 32 lanes
// contiguous.
//
// Work decomposition
//  * Elementwise phases (fused s-update + matvec + dot; AXPYs + max-norm): each
//    warp takes whole diagonals (32 contiguous slots), per-block partial sums
//    in FP64, and a fixed-order cross-block reduction that every block performs
//    identically, so all blocks take the same branch and results are
//    run-to-run deterministic.
//  * MIC(0) factor and both triangular solves: anti-diagonal wavefronts.  Warp
//    0 of block s owns strip s; lane l handles row 32s+l and at step t works on
//    diagonal t (backward: the mirrored diagonal), so the lower (upper)
//    neighbour's result arrives from lane l-1 (l+1) through a register
//    shuffle.  Operands stream through a shared-memory ring filled by bulk
//    asynchronous copies (cp.async.bulk, completion on an mbarrier), one
//    contiguous block of kSweepBlock diagonals per array.  Strips hand their
//    boundary row to the next strip through a halo row (one 8-byte store per
//    column, polled against a sentinel; no fence on the critical path).
//    Every cell runs
//    exactly the reference's arithmetic in a dependency-respecting order, so
//    the factor and the solves are bit-identical to the sequential loops.
//  * Phases are separated by a grid barrier of this file.
// Every wait is bounded: on timeout the status word gets FLAG_TIMEOUT, later
// waits stop waiting, the kernel runs to its end and the host reports an error.
#include <type_traits>

#include "ifl_device.cuh"

namespace ifl {

namespace {

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;
constexpr int kB = kSweepBlock;
constexpr long long kWaitLimit = 1ll << 22;      // ~1 s of flag polling
constexpr long long kMbarWaitLimit = 1ll << 20;  // try_wait suspends between polls
constexpr double kTau = 0.97, kSigma = 0.25, kTol = 1e-5;

template <typename F>
struct PcgArgs {
    SDIdx sd;
    const F *adiag, *ax, *ay;
    double *pc;
    F *pcf, *lx, *ly;
    const uint8_t *nb;
    double *r, *p;
    F *z, *sa, *sb, *as;
    double *partials;
    unsigned *barrier, *flags;
    double *halo_up, *halo_down;
    PcgOut *out;
    unsigned long long *iter_total;
    int mode, limit, pinned;
    int stages, stage_bytes;
};

// ------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
// 1-D bulk copy global -> shared (16-byte aligned, size a multiple of 16).
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool timed_out(const unsigned *flags) { return ld_volatile(flags) & FLAG_TIMEOUT; }

// Grid barrier: arrival counter + generation word, bounded wait.
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

// FP64 dot-product accumulation of stored values (explicit FMA for FP32 data).
__device__ __forceinline__ double dacc(double acc, double a, double b) { return acc + a * b; }
__device__ __forceinline__ double dacc(double acc, float a, float b) { return fma((double)a, (double)b, acc); }

// --------------------------------------------------------------- sweeps
// Per-warp shared-memory ring: `stages` buffers of stage_bytes, each holding
// kB diagonals (kB*32 slots) of up to five F arrays followed by the
// neighbour-bit bytes.  ii / ci count issued / consumed blocks over the whole
// kernel, so buffer = count % stages and mbarrier parity = (count/stages) & 1.
struct Ring {
    char *buf;
    uint64_t *bars;
    int stages, stage_bytes;
    unsigned ii, ci;
};

// Bounded wait for the block that ci refers to.
__device__ __forceinline__ void ring_wait(Ring &R, unsigned *flags) {
    const unsigned st = R.ci % R.stages, parity = (R.ci / R.stages) & 1u;
    long long n = 0;
    while (!mbar_try_wait(R.bars + st, parity)) {
        if (++n > kMbarWaitLimit || timed_out(flags)) {
            atomicOr(flags, FLAG_TIMEOUT);
            break;
        }
    }
    R.ci++;
}

// Streams of one sweep kind: KIND 0 factor (adiag, ax, ay), 1 forward (r, lx,
// ly, pcf), 2 backward (z, lx, ly, pcf, r).  Each stream owns a fixed 8-byte
// wide slot of the stage; the neighbour bits follow.
constexpr unsigned kSlotBytes = kB * 32 * 8;
constexpr unsigned kNbBytes = kB * 32;
constexpr int kStageBytes = 5 * kSlotBytes + kNbBytes;

template <int KIND, typename F>
struct Streams {
    static constexpr int n = KIND == 0 ? 3 : KIND == 1 ? 4 : 5;
    const void *src[5];
    unsigned esz[5];
    __device__ explicit Streams(const PcgArgs<F> &A) {
        for (int k = 0; k < 5; k++) esz[k] = sizeof(F);
        if (KIND == 0) {
            src[0] = A.adiag; src[1] = A.ax; src[2] = A.ay;
        } else if (KIND == 1) {
            src[0] = A.r; src[1] = A.lx; src[2] = A.ly; src[3] = A.pcf;
            esz[0] = 8;
        } else {
            src[0] = A.z; src[1] = A.lx; src[2] = A.ly; src[3] = A.pcf; src[4] = A.r;
            esz[4] = 8;
        }
        for (int k = n; k < 5; k++) src[k] = nullptr;
    }
};

// Issue the bulk copies of diagonal block `blk` of strip s (lane 0 only).
template <int KIND, typename F>
__device__ __forceinline__ void ring_issue(Ring &R, const PcgArgs<F> &A, const Streams<KIND, F> &St, int s,
                                           int blk) {
    const int D = A.sd.D;
    const int d0 = (KIND == 2) ? D - (blk + 1) * kB : blk * kB;
    const size_t off = ((size_t)s * D + d0) * 32;
    const unsigned st = R.ii % R.stages;
    char *dst = R.buf + (size_t)st * R.stage_bytes;
    uint64_t *bar = R.bars + st;
    unsigned total = kNbBytes;
    for (int k = 0; k < St.n; k++) total += kB * 32 * St.esz[k];
    fence_proxy_async_smem();
    mbar_expect_tx(bar, total);
    for (int k = 0; k < St.n; k++)
        bulk_g2s(dst + k * kSlotBytes, (const char *)St.src[k] + off * St.esz[k], kB * 32 * St.esz[k], bar);
    bulk_g2s(dst + 5 * kSlotBytes, A.nb + off, kNbBytes, bar);
    R.ii++;
}

// Halo rows hand a strip's boundary row to its neighbour strip.  An entry is
// the value's 8 bytes, or the sentinel while it has not been written; the
// producer writes each column once per sweep with one 8-byte store (no
// fence), the consumer polls and then puts the sentinel back.
constexpr unsigned long long kSentinel = ~0ull;

__device__ __forceinline__ double halo_take(double *slot, unsigned *flags) {
    volatile unsigned long long *p = (volatile unsigned long long *)slot;
    unsigned long long v = *p;
    long long n = 0;
    while (v == kSentinel) {
        if (++n > kWaitLimit || timed_out(flags)) {
            atomicOr(flags, FLAG_TIMEOUT);
            break;
        }
        v = *p;
    }
    *p = kSentinel;
    return __longlong_as_double((long long)v);
}
__device__ __forceinline__ void halo_put(double *slot, double v) {
    *(volatile unsigned long long *)slot = (unsigned long long)__double_as_longlong(v);
}

// One strip of a wavefront sweep.  Returns the lane's partial dot(z, r) for
// the backward solve.
template <int KIND, typename F>
__device__ double sweep_strip(const PcgArgs<F> &A, int s, Ring &R) {
    using V = typename std::conditional<KIND == 0, double, F>::type;
    const int lane = threadIdx.x & 31;
    const SDIdx sd = A.sd;
    const int W = sd.W, H = sd.H, D = sd.D, S = sd.S;
    const int y = s * 32 + lane;
    const bool rowok = y < H;
    const Streams<KIND, F> St(A);
    const int nblk = D / kB;
    // Backward sweeps run the top strip first: lane 31 takes from the strip
    // above, lane 0 hands its row to the strip below.
    const bool bwd = KIND == 2;
    const bool has_dep = bwd ? (s + 1 < S) : (s > 0);
    const bool producer = (lane == (bwd ? 0 : 31)) && (bwd ? s > 0 : s + 1 < S);
    double *halo_in = bwd ? A.halo_down + (size_t)(s + 1) * D : A.halo_up + (size_t)(s - 1) * D;
    double *halo_out = bwd ? A.halo_down + (size_t)s * D : A.halo_up + (size_t)s * D;
    double dot = 0.0;

    V prev = V(0);                   // result of the previous cell in sweep order
    F prev_a = F(0), prev_b = F(0);  // forward: lx, ly of that cell; factor: ax, ay

    if (lane == 0) {
        fence_proxy_async_global();  // generic-proxy writes before this sweep -> bulk copies
        const int pro = nblk < R.stages - 1 ? nblk : R.stages - 1;
        for (int b = 0; b < pro; b++) ring_issue<KIND, F>(R, A, St, s, b);
    }
    __syncwarp();
    for (int blk = 0; blk < nblk; blk++) {
        if (blk + R.stages - 1 < nblk) {
            __syncwarp();
            if (lane == 0) ring_issue<KIND, F>(R, A, St, s, blk + R.stages - 1);
        }
        // Boundary values of this block for the waiting lane: lane j fetches
        // the column the waiting lane works on at step j.
        double hv = 0.0;
        F ha = F(0), hb = F(0);
        if (has_dep && lane < kB) {
            const int xj = bwd ? D - 32 - blk * kB - lane : blk * kB + lane;
            if (xj >= 0 && xj < W) {
                if constexpr (KIND == 0) {
                    const size_t k = sd.slot(xj, s * 32 - 1);
                    ha = A.ax[k];
                    hb = A.ay[k];
                } else if constexpr (KIND == 1) {
                    hb = A.ly[sd.slot(xj, s * 32 - 1)];
                }
                hv = halo_take(halo_in + xj, A.flags);
            }
        }
        const unsigned st = R.ci % R.stages;
        ring_wait(R, A.flags);
        const char *sb = R.buf + (size_t)st * R.stage_bytes;
        const F *f0 = (const F *)sb;
        const double *d0 = (const double *)sb;
        const F *s1 = (const F *)(sb + kSlotBytes);
        const F *s2 = (const F *)(sb + 2 * kSlotBytes);
        const F *s3 = (const F *)(sb + 3 * kSlotBytes);
        const double *d4 = (const double *)(sb + 4 * kSlotBytes);
        const uint8_t *snb = (const uint8_t *)(sb + 5 * kSlotBytes);
#pragma unroll 4
        for (int j = 0; j < kB; j++) {
            const int t = blk * kB + j;
            const int d = bwd ? D - 1 - t : t;
            const int e = (bwd ? (kB - 1 - j) : j) * 32 + lane;  // slot inside the staged block
            const int x = d - lane;
            const bool active = rowok && x >= 0 && x < W;
            const size_t i = ((size_t)s * D + d) * 32 + lane;
            const uint8_t b = snb[e];
            const double hvj = __shfl_sync(0xffffffffu, hv, j);
            if constexpr (KIND == 0) {
                // buildPreconditioner (3-conjugate-gradients/Fluid.cpp:253-269)
                double pc_d = __shfl_up_sync(0xffffffffu, prev, 1);
                F ax_d = __shfl_up_sync(0xffffffffu, prev_a, 1);
                F ay_d = __shfl_up_sync(0xffffffffu, prev_b, 1);
                const F haj = __shfl_sync(0xffffffffu, ha, j), hbj = __shfl_sync(0xffffffffu, hb, j);
                if (lane == 0) {
                    pc_d = hvj;
                    ax_d = haj;
                    ay_d = hbj;
                }
                const F axv = s1[e], ayv = s2[e];
                V val = prev;
                if (active && (b & NB_SELF)) {
                    const double diag = (double)f0[e];
                    double ev = diag;
                    if (b & NB_LEFT) {
                        double px = (double)prev_a * prev;
                        double py = (double)prev_b * prev;
                        ev = ev - (px * px + kTau * px * py);
                    }
                    if (b & NB_DOWN) {
                        double px = (double)ax_d * pc_d;
                        double py = (double)ay_d * pc_d;
                        ev = ev - (py * py + kTau * px * py);
                    }
                    if (ev < kSigma * diag) ev = diag;
                    const double pcv = 1.0 / sqrt(ev);
                    A.pc[i] = pcv;
                    A.pcf[i] = (F)pcv;
                    A.lx[i] = (F)((double)axv * pcv);
                    A.ly[i] = (F)((double)ayv * pcv);
                    val = pcv;
                }
                prev = val;
                prev_a = axv;
                prev_b = ayv;
            } else if constexpr (KIND == 1) {
                // forward substitution (3-conjugate-gradients/Fluid.cpp:276-287)
                F q_d = __shfl_up_sync(0xffffffffu, prev, 1);
                F ly_d = __shfl_up_sync(0xffffffffu, prev_b, 1);
                const F hbj = __shfl_sync(0xffffffffu, hb, j);
                if (lane == 0) {
                    q_d = (F)hvj;
                    ly_d = hbj;
                }
                const F lxv = s1[e], lyv = s2[e];
                V val = prev;
                if (active && (b & NB_SELF)) {
                    F tt = (F)d0[e];
                    if (b & NB_LEFT) tt = tt - prev_a * prev;
                    if (b & NB_DOWN) tt = tt - ly_d * q_d;
                    val = tt * s3[e];
                    A.z[i] = val;
                }
                prev = val;
                prev_a = lxv;
                prev_b = lyv;
            } else {
                // backward substitution (3-conjugate-gradients/Fluid.cpp:289-303)
                F z_u = __shfl_down_sync(0xffffffffu, prev, 1);
                if (lane == 31) z_u = (F)hvj;
                V val = prev;
                if (active && (b & NB_SELF)) {
                    F tt = f0[e];
                    if (b & NB_RIGHT) tt = tt - s1[e] * prev;
                    if (b & NB_UP) tt = tt - s2[e] * z_u;
                    val = tt * s3[e];
                    A.z[i] = val;
                    if (b & NB_RED) dot = dacc(dot, (double)val, d4[e]);
                }
                prev = val;
            }
            if (producer && active) halo_put(halo_out + x, (double)prev);
        }
    }
    __syncwarp();
    return dot;
}

template <int KIND, typename F>
__device__ __forceinline__ double sweep(const PcgArgs<F> &A, Ring &R, bool sweeper) {
    if (!sweeper) return 0.0;
    return sweep_strip<KIND, F>(A, blockIdx.x, R);
}

template <typename F>
__global__ void __launch_bounds__(kThreads) pcg_kernel(PcgArgs<F> A) {
    extern __shared__ __align__(128) char smem_raw[];
    __shared__ double sm[kWarps + 1];
    const SDIdx sd = A.sd;
    const int W = sd.W, H = sd.H, D = sd.D;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rows = sd.S * D;  // diagonals of all strips
    const int gwarp = blockIdx.x * kWarps + warp, nwarps = gridDim.x * kWarps;
    const bool sweeper = warp == 0 && (int)blockIdx.x < sd.S;

    Ring R;
    R.bars = (uint64_t *)smem_raw;
    R.buf = smem_raw + 128;
    R.stages = A.stages;
    R.stage_bytes = A.stage_bytes;
    R.ii = R.ci = 0;
    if (sweeper) {
        if (lane == 0) {
            for (int k = 0; k < R.stages; k++) mbar_init(R.bars + k, 1);
            fence_mbar_init();
        }
        __syncwarp();
    }

    if (A.mode & PCG_FACTOR) {
        sweep<0, F>(A, R, sweeper);
        grid_barrier(A.barrier, A.flags);
    }
    if (!(A.mode & PCG_SOLVE)) return;

    // p = 0; maxError = |r|_inf   (3-conjugate-gradients/Fluid.cpp:350, 354)
    double mx = 0.0;
    for (int row = gwarp; row < rows; row += nwarps) {
        const size_t i = (size_t)row * 32 + lane;
        A.p[i] = 0.0;
        if (A.nb[i] & NB_RED) mx = smax(mx, fabs(A.r[i]));
    }
    block_store(mx, true, A.partials, 0, sm);
    // z = M^-1 r  (:351)
    sweep<1, F>(A, R, sweeper);
    grid_barrier(A.barrier, A.flags);
    double d = sweep<2, F>(A, R, sweeper);
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
            // s = z + beta*s (first iteration: s = z), then z' = A s and z'.s  (:361-362, 375)
            double dacc_ = 0.0;
            const F fbeta = (F)beta;
            for (int row = gwarp; row < rows; row += nwarps) {
                const int s = row / D, dd = row - s * D;
                const int x = dd - lane, y = s * 32 + lane;
                const size_t i = (size_t)row * 32 + lane;
                if (x < 0 || x >= W || y >= H) {
                    s_new[i] = F(0);
                    A.as[i] = F(0);
                    continue;
                }
                auto snew = [&](size_t k) -> F {
                    if (iter == 0) return A.z[k];
                    return (A.nb[k] & NB_RED) ? F(A.z[k] + s_old[k] * fbeta) : s_old[k];
                };
                const F sc = snew(i);
                F t = A.adiag[i] * sc;
                if (x > 0) t += A.ax[i - 32] * snew(i - 32);
                if (y > 0) {
                    const size_t k = lane > 0 ? i - 33 : sd.slot(x, y - 1);
                    t += A.ay[k] * snew(k);
                }
                if (x < W - 1) t += A.ax[i] * snew(i + 32);
                if (y < H - 1) t += A.ay[i] * snew(lane < 31 ? i + 33 : sd.slot(x, y + 1));
                s_new[i] = sc;
                A.as[i] = t;
                if (A.nb[i] & NB_RED) dacc_ = dacc(dacc_, t, sc);
            }
            block_store(dacc_, false, A.partials, 1, sm);
            grid_barrier(A.barrier, A.flags);
            const double alpha = sigma / grid_reduce(A.partials, 1, false, sm);
            // p += alpha s; r -= alpha z'; maxError = |r|_inf  (:363-366)
            mx = 0.0;
            for (int row = gwarp; row < rows; row += nwarps) {
                const size_t i = (size_t)row * 32 + lane;
                if (A.nb[i] & NB_RED) {
                    A.p[i] = A.p[i] + (double)s_new[i] * alpha;
                    const double rn = A.r[i] + (double)A.as[i] * -alpha;
                    A.r[i] = rn;
                    mx = smax(mx, fabs(rn));
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
            sweep<1, F>(A, R, sweeper);
            grid_barrier(A.barrier, A.flags);
            d = sweep<2, F>(A, R, sweeper);
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
        atomicAdd(A.iter_total, (unsigned long long)iterations);
    }
}

template <typename F>
int ring_stages() {
    return 4;
}
template <typename F>
int ring_stage_bytes() {
    return kStageBytes;
}
template <typename F>
size_t smem_bytes() {
    return 128 + (size_t)ring_stages<F>() * ring_stage_bytes<F>();
}

template <typename F>
int max_coresident() {
    static int cached = -1;
    if (cached < 0) {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaFuncSetAttribute(pcg_kernel<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes<F>());
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, pcg_kernel<F>, kThreads, smem_bytes<F>());
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
    A.sd = S.sd;
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
    A.halo_up = X.halo_up;
    A.halo_down = X.halo_down;
    A.flags = S.flags;
    A.out = X.out + (cfg.heat ? 1 : 0);
    A.iter_total = X.iter_total;
    A.mode = cfg.mode;
    A.limit = cfg.limit;
    A.pinned = cfg.pinned;
    A.stages = ring_stages<F>();
    A.stage_bytes = ring_stage_bytes<F>();
    int maxb = max_coresident<F>();
    if (maxb > X.max_blocks) maxb = X.max_blocks;
    if (maxb < S.sd.S) return cudaErrorInvalidConfiguration;  // one block per 32-row strip
    const long long slots = (long long)S.sd.total();
    int want = (int)((slots + kThreads * 4 - 1) / (kThreads * 4));
    if (want < S.sd.S) want = S.sd.S;
    int G = want < maxb ? want : maxb;
    if (blocks_used) *blocks_used = G;
    cudaMemsetAsync(X.barrier, 0, 2 * sizeof(unsigned), st);
    const size_t halo = (size_t)S.sd.S * S.sd.D * sizeof(double);
    cudaMemsetAsync(X.halo_up, 0xff, halo, st);  // every entry starts as the sentinel
    cudaMemsetAsync(X.halo_down, 0xff, halo, st);
    void *args[] = {&A};
    return cudaLaunchCooperativeKernel((const void *)pcg_kernel<F>, dim3(G), dim3(kThreads), args,
                                       smem_bytes<F>(), st);
}

template cudaError_t launch_pcg<double>(const Scene<double> &, const PcgScratch &, const PcgConfig &,
                                        cudaStream_t, int *);
template cudaError_t launch_pcg<float>(const Scene<float> &, const PcgScratch &, const PcgConfig &,
                                       cudaStream_t, int *);
template int pcg_max_blocks<double>();
template int pcg_max_blocks<float>();

}  // namespace ifl
