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
// contiguous.  r, p and A*s are FP64 in both forms; the FP32 form keeps an
// FP32 copy of r for the substitutions.
//
// Work decomposition
//  * Elementwise phases (fused s-update + matvec + dot; AXPYs + max-norm): each
//    warp takes whole diagonals (32 contiguous slots), FP64 partial sums per
//    block and a fixed-order cross-block reduction that every block performs
//    identically, so all blocks take the same branch and results are
//    run-to-run deterministic.
//  * MIC(0) factor and both triangular solves: anti-diagonal wavefronts.  A
//    block owns K consecutive 32-row strips, one per warp; lane l handles row
//    32s+l and at step t works on diagonal t (backward: the mirrored
//    diagonal), so the lower (upper) neighbour's value arrives from lane l-1
//    (l+1) through a register shuffle.  Operands stream through a per-warp
//    shared-memory ring filled by bulk asynchronous copies (cp.async.bulk,
//    completion on an mbarrier), one contiguous block of kSweepBlock diagonals
//    per array.  A strip hands its boundary row to the neighbouring strip
//    through a halo row: in shared memory between warps of one block, in
//    global memory between blocks; each entry is written once per sweep with
//    one 8-byte store and polled against a sentinel (no fences on the
//    critical path).  Every cell runs exactly the reference's arithmetic in a
//    dependency-respecting order, so the factor and the FP64 substitutions
//    are bit-identical to the sequential loops.
//  * Phases are separated by a grid barrier of this file.
// Every wait is bounded: on timeout the status word gets FLAG_TIMEOUT, later
// waits stop waiting, the kernel runs to its end and the host reports an error.
#include <type_traits>

#include "ifl_device.cuh"

namespace ifl {

namespace {

// Dynamic shared memory of the PCG kernel, addressed through this symbol so
// that every ring and halo access compiles to a shared-space instruction.
extern __shared__ __align__(128) char g_smem[];

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;
constexpr int kB = kSweepBlock;                  // diagonals per bulk-copy block
constexpr long long kWaitLimit = 1ll << 22;      // ~1 s of polling
constexpr long long kMbarWaitLimit = 1ll << 20;  // try_wait suspends between polls
constexpr double kTau = 0.97, kSigma = 0.25, kTol = 1e-5;
constexpr unsigned long long kSentinel = ~0ull;
constexpr unsigned FULL = 0xffffffffu;

template <typename F>
struct PcgArgs {
    SDIdx sd;
    const F *adiag, *ax, *ay;
    double *pc;
    F *mic;  // MIC record per slot: {lx, ly, pc, neighbour bits}
    const uint8_t *nb;
    double *r, *p, *as;
    F *rf;  // r in storage precision for the substitutions (== r when F is double)
    F *z, *sa, *sb;
    double *partials;
    unsigned *barrier, *flags;
    unsigned long long *halo;  // [2][S][D]: [0] rows handed upward, [1] rows handed downward
    PcgOut *out;
    unsigned long long *iter_total;
    int mode, limit, pinned;
    int K, stages;
};

// ------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
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
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) v = smax(v, __shfl_down_sync(FULL, v, o));
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

// ------------------------------------------------------------ halo words
__device__ __forceinline__ unsigned long long henc(double v) { return (unsigned long long)__double_as_longlong(v); }
__device__ __forceinline__ unsigned long long henc(float v) { return (unsigned long long)__float_as_uint(v); }
template <typename V> __device__ __forceinline__ V hdec(unsigned long long w);
template <> __device__ __forceinline__ double hdec<double>(unsigned long long w) {
    return __longlong_as_double((long long)w);
}
template <> __device__ __forceinline__ float hdec<float>(unsigned long long w) { return __uint_as_float((unsigned)w); }

// Halo rows: shared memory (relaxed, CTA scope) inside a block, global memory
// (relaxed, GPU scope) between blocks.  One 8-byte access is single-copy
// atomic, so a reader sees either the sentinel or the whole value.
struct Chan {
    unsigned soff;             // byte offset in g_smem when shared
    unsigned long long *g;     // global row when not shared
    bool shared, valid;
};
__device__ __forceinline__ unsigned long long hload(const Chan &c, int x) {
    unsigned long long v;
    if (c.shared)
        asm volatile("ld.relaxed.cta.shared.u64 %0, [%1];" : "=l"(v) : "r"(smem_u32(g_smem) + c.soff + 8u * x) : "memory");
    else
        asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(c.g + x) : "memory");
    return v;
}
__device__ __forceinline__ void hstore(const Chan &c, int x, unsigned long long v) {
    if (c.shared)
        asm volatile("st.relaxed.cta.shared.u64 [%0], %1;" ::"r"(smem_u32(g_smem) + c.soff + 8u * x), "l"(v) : "memory");
    else
        asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(c.g + x), "l"(v) : "memory");
}

// Take a halo word (bounded poll), then put the sentinel back for the next sweep.
__device__ __forceinline__ unsigned long long halo_take(const Chan &c, int x, unsigned long long pre,
                                                        unsigned *flags) {
    unsigned long long v = pre;
    long long n = 0;
    while (v == kSentinel) {
        v = hload(c, x);
        if (v != kSentinel) break;
        if (++n > kWaitLimit || timed_out(flags)) {
            atomicOr(flags, FLAG_TIMEOUT);
            v = 0;
            break;
        }
    }
    hstore(c, x, kSentinel);
    return v;
}

// --------------------------------------------------------------- sweeps
// Per-warp shared-memory ring: `stages` buffers, each holding kB diagonals
// (kB*32 slots) of the streams of one sweep kind, in three regions:
//   factor:   [adiag][ax][ay | neighbour bits]
//   forward:  [r]    [--][MIC record]
//   backward: [z]    [r] [MIC record]
// A MIC record is {lx, ly, pc, neighbour bits} for one slot (lx = aPlusX*pc,
// ly = aPlusY*pc, pc = precon, storage precision; written by the factor).
// ii / ci count issued / consumed blocks over the whole kernel, so buffer =
// count % stages and mbarrier parity = (count/stages) & 1.
template <typename F>
struct Ring {
    static constexpr unsigned kSlot = kB * 32 * sizeof(F);
    static constexpr unsigned kStageBytes = 6 * kSlot;
    unsigned buf;   // byte offset of this warp's stages in g_smem
    unsigned bars;  // byte offset of this warp's mbarriers in g_smem
    int stages;
    unsigned ii, ci;
    __device__ __forceinline__ uint64_t *bar(unsigned st) const { return (uint64_t *)(g_smem + bars) + st; }
};

template <typename F>
__device__ __forceinline__ void ring_wait(Ring<F> &R, unsigned *flags) {
    const unsigned st = R.ci % R.stages, parity = (R.ci / R.stages) & 1u;
    long long n = 0;
    while (!mbar_try_wait(R.bar(st), parity)) {
        if (++n > kMbarWaitLimit || timed_out(flags)) {
            atomicOr(flags, FLAG_TIMEOUT);
            break;
        }
    }
    R.ci++;
}

template <int KIND, typename F>
__device__ __forceinline__ void ring_issue(Ring<F> &R, const PcgArgs<F> &A, int s, int blk) {
    constexpr unsigned S1 = Ring<F>::kSlot;
    const int D = A.sd.D;
    const int d0 = (KIND == 2) ? D - (blk + 1) * kB : blk * kB;
    const size_t off = ((size_t)s * D + d0) * 32;
    const unsigned st = R.ii % R.stages;
    char *dst = g_smem + R.buf + st * Ring<F>::kStageBytes;
    uint64_t *bar = R.bar(st);
    if (KIND == 0) {
        mbar_expect_tx(bar, 3 * S1 + kB * 32);
        bulk_g2s(dst, A.adiag + off, S1, bar);
        bulk_g2s(dst + S1, A.ax + off, S1, bar);
        bulk_g2s(dst + 2 * S1, A.ay + off, S1, bar);
        bulk_g2s(dst + 3 * S1, A.nb + off, kB * 32, bar);
    } else if (KIND == 1) {
        mbar_expect_tx(bar, 5 * S1);
        bulk_g2s(dst, A.rf + off, S1, bar);
        bulk_g2s(dst + 2 * S1, A.mic + 4 * off, 4 * S1, bar);
    } else {
        mbar_expect_tx(bar, 6 * S1);
        bulk_g2s(dst, A.z + off, S1, bar);
        bulk_g2s(dst + S1, A.rf + off, S1, bar);
        bulk_g2s(dst + 2 * S1, A.mic + 4 * off, 4 * S1, bar);
    }
    R.ii++;
}

__device__ __forceinline__ void ld4(const float *p, float &a, float &b, float &c, float &d) {
    const float4 v = *(const float4 *)p;
    a = v.x; b = v.y; c = v.z; d = v.w;
}
__device__ __forceinline__ void ld4(const double *p, double &a, double &b, double &c, double &d) {
    const double2 v0 = *(const double2 *)p, v1 = *(const double2 *)(p + 2);
    a = v0.x; b = v0.y; c = v1.x; d = v1.y;
}
__device__ __forceinline__ void st4(float *p, float a, float b, float c, float d) {
    *(float4 *)p = make_float4(a, b, c, d);
}
__device__ __forceinline__ void st4(double *p, double a, double b, double c, double d) {
    *(double2 *)p = make_double2(a, b);
    *(double2 *)(p + 2) = make_double2(c, d);
}
__device__ __forceinline__ unsigned nb_of(float w) { return __float_as_uint(w); }
__device__ __forceinline__ unsigned nb_of(double w) { return (unsigned)__double_as_longlong(w); }
__device__ __forceinline__ float nb_word(unsigned b, float) { return __uint_as_float(b); }
__device__ __forceinline__ double nb_word(unsigned b, double) { return __longlong_as_double((long long)b); }

// One strip of a wavefront sweep.  `in` is the halo row written by the
// neighbouring strip this one depends on (nullptr: none), `out` the row this
// strip hands on (nullptr: none).  Each sub-block of kHB steps first stages
// its operands from the ring into registers, then runs the dependency chain
// (registers and shuffles only), then issues its stores.  Returns the lane's
// partial dot(z, r) for the backward solve.
template <int KIND, typename F>
__device__ double sweep_strip(const PcgArgs<F> &A, int s, Ring<F> &R, const Chan in, const Chan out) {
    using V = typename std::conditional<KIND == 0, double, F>::type;
    constexpr int kHB = sizeof(F) == 8 ? 4 : 8;
    constexpr bool bwd = KIND == 2;
    constexpr unsigned S1 = Ring<F>::kSlot;
    const int lane = threadIdx.x & 31;
    const SDIdx sd = A.sd;
    const int W = sd.W, H = sd.H, D = sd.D;
    const int y = s * 32 + lane;
    const bool rowok = y < H;
    const int nblk = D / kB;
    const bool has_in = in.valid;
    const bool producer = out.valid && lane == (bwd ? 0 : 31);
    double dot = 0.0;

    V prev = V(0);                   // result of the previous cell in sweep order
    F prev_a = F(0), prev_b = F(0);  // forward: lx, ly of that cell; factor: ax, ay

    // Halo prefetch: lane l < kHB holds the word of the column that the
    // waiting lane (0 forward, 31 backward) reaches at step t0 + l.
    unsigned long long hpre = kSentinel;
    F spre_a = F(0), spre_b = F(0);
    auto halo_col = [&](int t) { return bwd ? D - 32 - t : t; };
    auto prefetch = [&](int t0) {
        hpre = kSentinel;
        if (has_in && lane < kHB) {
            const int xc = halo_col(t0 + lane);
            if (xc >= 0 && xc < W) {
                hpre = hload(in, xc);
                if constexpr (KIND == 0) {
                    const size_t k = sd.slot(xc, s * 32 - 1);
                    spre_a = A.ax[k];
                    spre_b = A.ay[k];
                } else if constexpr (KIND == 1) {
                    F a, b, c, d;
                    ld4(A.mic + 4 * sd.slot(xc, s * 32 - 1), a, b, c, d);
                    spre_b = b;  // ly of the cell below
                }
            }
        }
    };

    if (lane == 0) {
        fence_proxy_async_global();  // generic-proxy writes before this sweep -> bulk copies
        const int pro = nblk < R.stages - 1 ? nblk : R.stages - 1;
        for (int b = 0; b < pro; b++) ring_issue<KIND, F>(R, A, s, b);
    }
    prefetch(0);
    __syncwarp();
    for (int blk = 0; blk < nblk; blk++) {
        if (blk + R.stages - 1 < nblk) {
            __syncwarp();
            if (lane == 0) ring_issue<KIND, F>(R, A, s, blk + R.stages - 1);
        }
        const unsigned st = R.ci % R.stages;
        ring_wait(R, A.flags);
        const char *sbuf = g_smem + R.buf + st * Ring<F>::kStageBytes;
        const F *g0 = (const F *)sbuf;
        const F *g1 = (const F *)(sbuf + S1);
        const F *g2 = (const F *)(sbuf + 2 * S1);
        const uint8_t *gnb = (const uint8_t *)(sbuf + 3 * S1);
        for (int sub = 0; sub < kB / kHB; sub++) {
            const int t0 = blk * kB + sub * kHB;
            // halo words of this sub-block, then the next sub-block's prefetch
            V hv = V(0);
            F ha = F(0), hb = F(0);
            if (has_in && lane < kHB) {
                const int xc = halo_col(t0 + lane);
                if (xc >= 0 && xc < W) {
                    hv = hdec<V>(halo_take(in, xc, hpre, A.flags));
                    ha = spre_a;
                    hb = spre_b;
                }
            }
            prefetch(t0 + kHB);
            // stage this sub-block's operands in registers
            F o0[kHB], o1[kHB], o2[kHB], o3[kHB], o4[kHB];
            unsigned ob[kHB];
            V hvv[kHB];
            F hav[kHB], hbv[kHB];
#pragma unroll
            for (int jj = 0; jj < kHB; jj++) {
                const int j = sub * kHB + jj;
                const int e = (bwd ? (kB - 1 - j) : j) * 32 + lane;  // slot inside the staged block
                if constexpr (KIND == 0) {
                    o0[jj] = g0[e];
                    o1[jj] = g1[e];
                    o2[jj] = g2[e];
                    ob[jj] = gnb[e];
                    o3[jj] = o4[jj] = F(0);
                } else if constexpr (KIND == 1) {
                    F w3;
                    o0[jj] = g0[e];
                    ld4(g2 + 4 * e, o1[jj], o2[jj], o3[jj], w3);
                    ob[jj] = nb_of(w3);
                    o4[jj] = F(0);
                } else {
                    F w3;
                    o0[jj] = g0[e];
                    o4[jj] = g1[e];
                    ld4(g2 + 4 * e, o1[jj], o2[jj], o3[jj], w3);
                    ob[jj] = nb_of(w3);
                }
                hvv[jj] = __shfl_sync(FULL, hv, jj);
                hav[jj] = __shfl_sync(FULL, ha, jj);
                hbv[jj] = __shfl_sync(FULL, hb, jj);
            }
            // dependency chain
            V res[kHB];
#pragma unroll
            for (int jj = 0; jj < kHB; jj++) {
                const unsigned b = ob[jj];
                V val;
                if constexpr (KIND == 0) {
                    // buildPreconditioner (3-conjugate-gradients/Fluid.cpp:253-269)
                    double pc_d = __shfl_up_sync(FULL, prev, 1);
                    F ax_d = __shfl_up_sync(FULL, prev_a, 1);
                    F ay_d = __shfl_up_sync(FULL, prev_b, 1);
                    if (lane == 0) {
                        pc_d = hvv[jj];
                        ax_d = hav[jj];
                        ay_d = hbv[jj];
                    }
                    const double diag = (double)o0[jj];
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
                    val = 1.0 / sqrt(ev);
                    prev_a = o1[jj];
                    prev_b = o2[jj];
                } else if constexpr (KIND == 1) {
                    // forward substitution (3-conjugate-gradients/Fluid.cpp:276-287)
                    const F q_sh = __shfl_up_sync(FULL, prev, 1);
                    const F ly_sh = __shfl_up_sync(FULL, prev_b, 1);
                    const F q_d = lane == 0 ? hvv[jj] : q_sh;
                    const F ly_d = lane == 0 ? hbv[jj] : ly_sh;
                    F tt = o0[jj];
                    tt = (b & NB_LEFT) ? tt - prev_a * prev : tt;
                    tt = (b & NB_DOWN) ? tt - ly_d * q_d : tt;
                    val = tt * o3[jj];
                    prev_a = o1[jj];
                    prev_b = o2[jj];
                } else {
                    // backward substitution (3-conjugate-gradients/Fluid.cpp:289-303)
                    const F z_sh = __shfl_down_sync(FULL, prev, 1);
                    const F z_u = lane == 31 ? hvv[jj] : z_sh;
                    F tt = o0[jj];
                    tt = (b & NB_RIGHT) ? tt - o1[jj] * prev : tt;
                    tt = (b & NB_UP) ? tt - o2[jj] * z_u : tt;
                    val = tt * o3[jj];
                }
                res[jj] = val;
                prev = val;
            }
            // stores
#pragma unroll
            for (int jj = 0; jj < kHB; jj++) {
                const int t = t0 + jj;
                const int d = bwd ? D - 1 - t : t;
                const int x = d - lane;
                const bool active = rowok && x >= 0 && x < W;
                const size_t i = ((size_t)s * D + d) * 32 + lane;
                const unsigned b = ob[jj];
                if (active) {
                    if constexpr (KIND == 0) {
                        const bool self = b & NB_SELF;
                        const double pcv = res[jj];
                        if (self) A.pc[i] = pcv;
                        st4(A.mic + 4 * i, self ? (F)((double)o1[jj] * pcv) : F(0),
                            self ? (F)((double)o2[jj] * pcv) : F(0), self ? (F)pcv : F(0), nb_word(b, F(0)));
                    } else {
                        if (b & NB_SELF) {
                            A.z[i] = res[jj];
                            if (KIND == 2 && (b & NB_RED)) dot = fma((double)res[jj], (double)o4[jj], dot);
                        }
                    }
                    if (producer) hstore(out, x, henc(res[jj]));
                }
            }
        }
    }
    __syncwarp();
    return dot;
}

// Sweep of all strips of this block; the halo rows between its own warps live
// in shared memory, those to neighbouring blocks in global memory.
// hsm_off: byte offset in g_smem of the K-1 shared halo rows (D words each).
template <int KIND, typename F>
__device__ double sweep(const PcgArgs<F> &A, Ring<F> &R, unsigned hsm_off, int nstrips_blk) {
    const int w = threadIdx.x >> 5;
    if (w >= nstrips_blk) return 0.0;
    const SDIdx sd = A.sd;
    const int s = blockIdx.x * A.K + w;
    const size_t D = sd.D;
    unsigned long long *up = A.halo, *down = A.halo + (size_t)sd.S * D;
    auto smem_row = [&](int k) { return Chan{hsm_off + 8u * (unsigned)(k * D), nullptr, true, true}; };
    auto glob_row = [&](unsigned long long *row) { return Chan{0u, row, false, true}; };
    Chan in{0u, nullptr, false, false}, out{0u, nullptr, false, false};
    if (KIND != 2) {  // rows travel upward: strip s takes from s-1, gives to s+1
        if (s > 0) in = (w > 0) ? smem_row(w - 1) : glob_row(up + (size_t)(s - 1) * D);
        if (s + 1 < sd.S) out = (w + 1 < nstrips_blk) ? smem_row(w) : glob_row(up + (size_t)s * D);
    } else {          // downward: strip s takes from s+1, gives to s-1
        if (s + 1 < sd.S) in = (w + 1 < nstrips_blk) ? smem_row(w) : glob_row(down + (size_t)(s + 1) * D);
        if (s > 0) out = (w > 0) ? smem_row(w - 1) : glob_row(down + (size_t)s * D);
    }
    return sweep_strip<KIND, F>(A, s, R, in, out);
}

template <typename F>
__global__ void __launch_bounds__(kThreads, 1) pcg_kernel(PcgArgs<F> A) {
    __shared__ double sm[kWarps + 1];
    const SDIdx sd = A.sd;
    const int W = sd.W, H = sd.H, D = sd.D;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rows = sd.S * D;  // diagonals of all strips
    const int gwarp = blockIdx.x * kWarps + warp, nwarps = gridDim.x * kWarps;
    int nstrips_blk = sd.S - (int)blockIdx.x * A.K;
    nstrips_blk = nstrips_blk < 0 ? 0 : (nstrips_blk > A.K ? A.K : nstrips_blk);
    constexpr bool kF32 = !std::is_same<F, double>::value;

    // shared memory: mbarriers | halo rows between this block's strips | rings
    const size_t nh = (size_t)(A.K > 1 ? A.K - 1 : 0) * D;
    const unsigned hsm_off = 32u * A.K;
    const unsigned rings = (unsigned)(((32 * A.K + nh * 8 + 127) / 128) * 128);
    Ring<F> R;
    R.bars = 32u * warp;
    R.buf = rings + (unsigned)warp * A.stages * Ring<F>::kStageBytes;
    R.stages = A.stages;
    R.ii = R.ci = 0;
    for (size_t k = threadIdx.x; k < nh; k += kThreads) ((unsigned long long *)(g_smem + hsm_off))[k] = kSentinel;
    if (warp < nstrips_blk && lane == 0) {
        for (int k = 0; k < R.stages; k++) mbar_init(R.bar(k), 1);
        fence_mbar_init();
    }
    __syncthreads();

    if (A.mode & PCG_FACTOR) {
        sweep<0, F>(A, R, hsm_off, nstrips_blk);
        grid_barrier(A.barrier, A.flags);
    }
    if (!(A.mode & PCG_SOLVE)) return;

    // p = 0; maxError = |r|_inf   (3-conjugate-gradients/Fluid.cpp:350, 354)
    double mx = 0.0;
    for (int row = gwarp; row < rows; row += nwarps) {
        const size_t i = (size_t)row * 32 + lane;
        A.p[i] = 0.0;
        if (kF32) A.rf[i] = (F)A.r[i];
        if (A.nb[i] & NB_RED) mx = smax(mx, fabs(A.r[i]));
    }
    block_store(mx, true, A.partials, 0, sm);
    if (kF32) grid_barrier(A.barrier, A.flags);  // FP32 copy of r complete
    // z = M^-1 r  (:351)
    sweep<1, F>(A, R, hsm_off, nstrips_blk);
    grid_barrier(A.barrier, A.flags);
    double d = sweep<2, F>(A, R, hsm_off, nstrips_blk);
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
            double dacc = 0.0;
            const F fbeta = (F)beta;
            for (int row = gwarp; row < rows; row += nwarps) {
                const int s = row / D, dd = row - s * D;
                const int x = dd - lane, y = s * 32 + lane;
                const size_t i = (size_t)row * 32 + lane;
                if (x < 0 || x >= W || y >= H) {
                    s_new[i] = F(0);
                    A.as[i] = 0.0;
                    continue;
                }
                auto snew = [&](size_t k) -> F {
                    if (iter == 0) return A.z[k];
                    return (A.nb[k] & NB_RED) ? F(A.z[k] + s_old[k] * fbeta) : s_old[k];
                };
                // FP64 accumulation: with FP32 storage every product is exact,
                // so the operator the recurrences see is the same every iteration.
                const F sc = snew(i);
                double t = (double)A.adiag[i] * (double)sc;
                if (x > 0) t += (double)A.ax[i - 32] * (double)snew(i - 32);
                if (y > 0) {
                    const size_t k = lane > 0 ? i - 33 : sd.slot(x, y - 1);
                    t += (double)A.ay[k] * (double)snew(k);
                }
                if (x < W - 1) t += (double)A.ax[i] * (double)snew(i + 32);
                if (y < H - 1) t += (double)A.ay[i] * (double)snew(lane < 31 ? i + 33 : sd.slot(x, y + 1));
                s_new[i] = sc;
                A.as[i] = t;
                if (A.nb[i] & NB_RED) dacc += t * (double)sc;
            }
            block_store(dacc, false, A.partials, 1, sm);
            grid_barrier(A.barrier, A.flags);
            const double alpha = sigma / grid_reduce(A.partials, 1, false, sm);
            // p += alpha s; r -= alpha z'; maxError = |r|_inf  (:363-366)
            mx = 0.0;
            for (int row = gwarp; row < rows; row += nwarps) {
                const size_t i = (size_t)row * 32 + lane;
                if (A.nb[i] & NB_RED) {
                    A.p[i] = A.p[i] + (double)s_new[i] * alpha;
                    const double rn = A.r[i] + A.as[i] * -alpha;
                    A.r[i] = rn;
                    if (kF32) A.rf[i] = (F)rn;
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
            sweep<1, F>(A, R, hsm_off, nstrips_blk);
            grid_barrier(A.barrier, A.flags);
            d = sweep<2, F>(A, R, hsm_off, nstrips_blk);
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

// Strips per block: the rings of the sweeping warps and the halo rows between
// them must fit in shared memory.
template <typename F>
int strips_per_block() {
    return sizeof(F) == 8 ? 2 : 4;
}
constexpr int kStages = 3;
template <typename F>
size_t smem_bytes(int K, int D) {
    const size_t nh = (size_t)(K > 1 ? K - 1 : 0) * D;
    return ((32 * (size_t)K + nh * 8 + 127) / 128) * 128 + (size_t)K * kStages * Ring<F>::kStageBytes;
}

template <typename F>
int max_coresident(size_t smem) {
    static size_t cached_smem = 0;
    static int cached = -1;
    if (cached < 0 || cached_smem != smem) {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaFuncSetAttribute(pcg_kernel<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, pcg_kernel<F>, kThreads, smem);
        cached = sms * (per > 2 ? 2 : per);
        cached_smem = smem;
    }
    return cached;
}

}  // namespace

template <typename F>
int pcg_max_blocks() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return 2 * sms;
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
    A.mic = S.mic;
    A.nb = S.nb;
    A.r = S.r;
    A.p = S.p;
    A.as = S.as;
    A.rf = S.rf;
    A.z = S.z;
    A.sa = S.sa;
    A.sb = S.sb;
    A.partials = X.partials;
    A.barrier = X.barrier;
    A.halo = X.halo;
    A.flags = S.flags;
    A.out = X.out + (cfg.heat ? 1 : 0);
    A.iter_total = X.iter_total;
    A.mode = cfg.mode;
    A.limit = cfg.limit;
    A.pinned = cfg.pinned;
    A.K = strips_per_block<F>();
    if (A.K > S.sd.S) A.K = S.sd.S;
    A.stages = kStages;
    const size_t smem = smem_bytes<F>(A.K, S.sd.D);
    int maxb = max_coresident<F>(smem);
    if (maxb > X.max_blocks) maxb = X.max_blocks;
    const int need = (S.sd.S + A.K - 1) / A.K;  // blocks that own strips
    if (maxb < need) return cudaErrorInvalidConfiguration;
    const long long slots = (long long)S.sd.total();
    int want = (int)((slots + kThreads * 4 - 1) / (kThreads * 4));
    if (want < need) want = need;
    int G = want < maxb ? want : maxb;
    if (blocks_used) *blocks_used = G;
    cudaMemsetAsync(X.barrier, 0, 2 * sizeof(unsigned), st);
    cudaMemsetAsync(X.halo, 0xff, 2 * (size_t)S.sd.S * S.sd.D * sizeof(unsigned long long), st);
    void *args[] = {&A};
    return cudaLaunchCooperativeKernel((const void *)pcg_kernel<F>, dim3(G), dim3(kThreads), args, smem, st);
}

template cudaError_t launch_pcg<double>(const Scene<double> &, const PcgScratch &, const PcgConfig &,
                                        cudaStream_t, int *);
template cudaError_t launch_pcg<float>(const Scene<float> &, const PcgScratch &, const PcgConfig &,
                                       cudaStream_t, int *);
template int pcg_max_blocks<double>();
template int pcg_max_blocks<float>();

}  // namespace ifl
