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
//    completion on an mbarrier), one contiguous block of kB diagonals
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
#include <algorithm>
#include <functional>
#include <cstring>
#include <type_traits>
#include <vector>

#include "ifl_device.cuh"

namespace ifl {

namespace {

// Dynamic shared memory of the PCG kernel, addressed through this symbol so
// that every ring and halo access compiles to a shared-space instruction.
extern __shared__ __align__(128) char g_smem[];

// Threads per block: 512 for a scene that has the GPU to itself, 256 in the
// compact launch used when many scenes run concurrently.
constexpr int kMaxWarps = 16;
constexpr int kChunk = kPcgChunk;  // diagonals per reduction chunk of the elementwise phases
// Diagonals per bulk-copy block of a sweep ring (the layout's padding unit).
// Halving it lets 16 single-warp blocks share an SM, which measured slower on
// full batch steps (30.7 M against 36.5 M cell-steps/s): the second warp of a
// 64-thread block, which works only in the elementwise passes, pays for more.
constexpr int kB = kSweepBlock;
// Default polls of a halo-word or barrier wait (about a second); the host may
// set another limit per solve (PcgConfig::wait_limit).  The mbarrier waits of
// the bulk-copy rings keep their own fixed limit: they wait for copies this
// warp issued from this GPU's memory, which always complete, and a timed-out
// sweep still waits for every copy it issued before it leaves.
constexpr long long kWaitLimit = 1ll << 22;
constexpr long long kMbarWaitLimit = 1ll << 20;  // try_wait suspends between polls
constexpr double kTau = 0.97, kSigma = 0.25, kTol = 1e-5;
constexpr unsigned long long kSentinel = ~0ull;
constexpr unsigned FULL = 0xffffffffu;

// Status words a wait checks: the scene's own and one shared by every scene
// of a batched launch (the same word for a single-scene launch).  A timed-out
// wait marks both, so every later wait of the launch stops waiting.
struct Flags {
    unsigned *scene, *all;
    long long limit;  // polls of one halo or barrier wait before it gives up
};

// The blocks that solve one scene: ranks 0..size-1, their barrier words and
// the per-block partial sums.  A single-scene launch is one team of the whole
// grid.
struct Team {
    int rank, size;
    unsigned *barrier;
    double *partials;
};

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
    unsigned *barrier;
    Flags fl;
    unsigned long long *halo;  // [2][S][D]: [0] rows handed upward, [1] rows handed downward
    PcgOut *out;
    unsigned long long *iter_total;
    int mode, limit, pinned;
    int K, stages;
    int rowsum_zero;  // 1: pressure matrix (rows sum to zero), 0: heat matrix
    int all_red;      // 1: every cell takes part in the dot products and AXPYs (unmasked solves)
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

__device__ __forceinline__ bool timed_out(const Flags &f) {
    return (ld_volatile(f.scene) | ld_volatile(f.all)) & FLAG_TIMEOUT;
}
__device__ __forceinline__ void set_timeout(const Flags &f) {
    atomicOr(f.scene, FLAG_TIMEOUT);
    if (f.all != f.scene) atomicOr(f.all, FLAG_TIMEOUT);
}

// Team barrier: arrival counter + generation word, bounded wait.  A team of
// one block needs only the block barrier.
__device__ void team_barrier(const Team &T, const Flags &fl) {
    __syncthreads();
    if (T.size == 1) return;
    if (threadIdx.x == 0) {
        unsigned *bar = T.barrier;
        unsigned g = ld_volatile(bar + 1);
        __threadfence();
        unsigned arrived = atomicAdd(bar, 1u);
        if (arrived == (unsigned)T.size - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            long long n = 0;
            while (ld_volatile(bar + 1) == g) {
                if (++n > fl.limit || timed_out(fl)) {
                    set_timeout(fl);
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

// ------------------------------------------------------------ halo words
__device__ __forceinline__ unsigned long long henc(double v) { return (unsigned long long)__double_as_longlong(v); }
__device__ __forceinline__ unsigned long long henc(float v) { return (unsigned long long)__float_as_uint(v); }
template <typename V> __device__ __forceinline__ V hdec(unsigned long long w);
template <> __device__ __forceinline__ double hdec<double>(unsigned long long w) {
    return __longlong_as_double((long long)w);
}
template <> __device__ __forceinline__ float hdec<float>(unsigned long long w) { return __uint_as_float((unsigned)w); }

// Halo rows: shared memory between warps of one block, global memory between
// blocks.  A channel holds the row's generic address, so one instruction
// serves both spaces (relaxed, GPU scope; stronger than a shared row needs).
// One 8-byte access is single-copy atomic, so a reader sees either the
// sentinel or the whole word.  A halo word carries its value itself, so no
// other memory access has to be ordered around it: the asm statements are
// volatile (kept, in program order) but do not clobber memory.  Loads and
// stores are predicated inside the asm: a sweep step never branches around a
// halo access.
struct Chan {
    unsigned long long *row;  // generic address of the row (word x at row + x)
    bool valid;
};
__device__ __forceinline__ unsigned long long hload(const Chan &c, int x) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.u64 %0, [%1];" : "=l"(v) : "l"(c.row + x));
    return v;
}
// The word at x where p holds, else `other`.
__device__ __forceinline__ unsigned long long hload_if(const Chan &c, int x, bool p, unsigned long long other) {
    unsigned long long v = other;
    asm volatile("{\n .reg .pred q;\n setp.ne.u32 q, %2, 0;\n @q ld.relaxed.gpu.u64 %0, [%1];\n}\n"
                 : "+l"(v)
                 : "l"(c.row + x), "r"((unsigned)p));
    return v;
}
__device__ __forceinline__ void hstore_if(const Chan &c, int x, unsigned long long v, bool p) {
    asm volatile("{\n .reg .pred q;\n setp.ne.u32 q, %2, 0;\n @q st.relaxed.gpu.u64 [%0], %1;\n}\n" ::"l"(c.row + x),
                 "l"(v), "r"((unsigned)p));
}

// Halo words of one sub-block: lane l < n needs the word at column xs[l]
// (need), prefetched in w.  Lanes whose word is still the sentinel poll it
// (bounded; the whole warp loops together, only in this slow path); then the
// sentinel goes back for the next sweep.  A timed-out wait yields 0.
__device__ __forceinline__ unsigned long long halo_take_warp(const Chan &c, int x, bool need, unsigned long long w,
                                                             const Flags &flags) {
    if (__any_sync(FULL, need && w == kSentinel)) {
        long long n = 0;
        bool given_up = false;
        for (;;) {
            const bool wait = need && w == kSentinel && !given_up;
            if (!__any_sync(FULL, wait)) break;
            if (wait) {
                w = hload(c, x);
                if (w == kSentinel && (++n > flags.limit || timed_out(flags))) {
                    set_timeout(flags);
                    given_up = true;
                }
            }
        }
        if (given_up) w = 0ull;
    }
    hstore_if(c, x, kSentinel, need);
    return w;
}

// --------------------------------------------------------------- sweeps
// Per-warp shared-memory ring: `stages` buffers, each holding kB diagonals
// (kB*32 slots) of the streams of one sweep kind, in three regions:
//   factor:   [adiag][ax][ay | neighbour bits]
//   forward:  [r]    [--][MIC record]
//   backward: [z]    [--][MIC record]
// A MIC record is {lx, ly, pc, neighbour bits} for one slot (lx = aPlusX*pc,
// ly = aPlusY*pc, pc = precon, storage precision; written by the factor).
// ii / ci count issued / consumed blocks over the whole kernel, so buffer =
// count % stages and mbarrier parity = (count/stages) & 1.
// A ring is `dead` once one of its mbarrier waits ran out (a copy that never
// completed): it then issues and waits for nothing more.
//
// The same warp state carries the staging area of the elementwise passes:
// sbuf/sbytes (this warp's share of the block's ring memory, idle outside the
// sweeps), the staging mbarrier at sbar and its completed phases sphase.
template <typename F>
struct Ring {
    static constexpr unsigned kSlot = kB * 32 * sizeof(F);
    static constexpr unsigned kStageBytes = 6 * kSlot;
    unsigned buf;   // byte offset of this warp's stages in g_smem
    unsigned bars;  // byte offset of this warp's mbarriers in g_smem
    int stages;
    unsigned ii, ci;
    bool dead;
    unsigned sbuf, sbytes, sbar, sphase;
    bool sdead;
    __device__ __forceinline__ uint64_t *bar(unsigned st) const { return (uint64_t *)(g_smem + bars) + st; }
    __device__ __forceinline__ uint64_t *stage_bar() const { return (uint64_t *)(g_smem + sbar); }
};

// Wait for the oldest issued block.  A timeout elsewhere in the launch does not
// shorten this wait: the copy was issued by this warp from this GPU's memory
// and completes, and a stage is re-armed only after its previous phase
// completed, so the ring never leaves a bulk copy writing shared memory behind
// (every sweep consumes every block it issued).
template <typename F>
__device__ __forceinline__ void ring_wait(Ring<F> &R, const Flags &flags) {
    const unsigned st = R.ci % R.stages, parity = (R.ci / R.stages) & 1u;
    long long n = 0;
    while (!R.dead && !mbar_try_wait(R.bar(st), parity)) {
        if (++n > kMbarWaitLimit) {
            set_timeout(flags);
            R.dead = true;
        }
    }
    R.dead = __any_sync(FULL, R.dead);  // the whole warp issues and waits alike
    R.ci++;
}

template <int KIND, typename F>
__device__ __forceinline__ void ring_issue(Ring<F> &R, const PcgArgs<F> &A, int s, int blk) {
    if (R.dead) {
        R.ii++;
        return;
    }
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
        mbar_expect_tx(bar, 5 * S1);
        bulk_g2s(dst, A.z + off, S1, bar);
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
// Float-float numbers (hi + lo, |lo| <= ulp(hi)/2): an exact product of two
// floats and a sum with an error-free two-sum of the high parts (Knuth's
// TwoSum; the library is compiled without contraction, so these stay exact).
struct FF {
    float hi, lo;
};
__device__ __forceinline__ FF ff_prod(float a, float b) {
    const float p = a * b;
    return FF{p, fmaf(a, b, -p)};
}
__device__ __forceinline__ FF ff_add(FF x, FF y) {
    const float s = x.hi + y.hi;
    const float bb = s - x.hi;
    const float err = (x.hi - (s - bb)) + (y.hi - bb);
    const float lo = err + x.lo + y.lo;
    const float hi = s + lo;
    return FF{hi, lo - (hi - s)};
}

// t - a*b: one fused multiply-add in the FP32 form; two roundings in FP64, as
// the reference computes it (the FP64 path must stay bit-identical).
__device__ __forceinline__ float msub(float t, float a, float b) { return fmaf(-a, b, t); }
__device__ __forceinline__ double msub(double t, double a, double b) { return t - a * b; }
__device__ __forceinline__ unsigned nb_of(float w) { return __float_as_uint(w); }
__device__ __forceinline__ unsigned nb_of(double w) { return (unsigned)__double_as_longlong(w); }
__device__ __forceinline__ float nb_word(unsigned b, float) { return __uint_as_float(b); }
__device__ __forceinline__ double nb_word(unsigned b, double) { return __longlong_as_double((long long)b); }

// One strip of a wavefront sweep.  `in` is the halo row written by the
// neighbouring strip this one depends on (IN says at compile time whether it
// exists: a strip without one carries no halo code), `out` the row this strip
// hands on (valid or not).  Each sub-block of kHB steps stages its operands
// from the ring into registers, takes the sub-block's halo words (lanes
// 0..kHB-1 one column each, prefetched one sub-block ahead), runs the
// dependency chain (registers and shuffles only; the handing-on lane stores
// each boundary value as soon as the chain computes it) and issues its
// stores.
//
// Halo words: the FP32 forward sweep hands over the pair (q, aPlusY*precon)
// of the strip's top cell packed in one 8-byte word, so the strip above needs
// no load of its lower neighbour's MIC(0) record; the other sweeps hand over
// the value alone (the factor and the FP64 forward sweep load the lower
// neighbour's coefficients with the prefetch).
template <int KIND, typename F, bool IN>
__device__ void sweep_strip(const PcgArgs<F> &A, int s, Ring<F> &R, const Chan in, const Chan out) {
    using V = typename std::conditional<KIND == 0, double, F>::type;
    constexpr int kHB = sizeof(F) == 8 ? 4 : 8;
    constexpr bool bwd = KIND == 2;
    constexpr bool kPair = KIND == 1 && sizeof(F) == 4;  // packed (q, ly) words
    constexpr unsigned S1 = Ring<F>::kSlot;
    const int lane = threadIdx.x & 31;
    const SDIdx sd = A.sd;
    const int W = sd.W, H = sd.H, D = sd.D;
    const int y = s * 32 + lane;
    const bool rowok = y < H;
    const int nblk = D / kB;
    const bool producer = out.valid && lane == (bwd ? 0 : 31);
    // pointers in registers for the whole sweep
    F *const zout = A.z;
    F *const micp = A.mic;
    double *const pcp = A.pc;
    const F *const axp = A.ax;
    const F *const ayp = A.ay;

    V prev = V(0);                   // result of the previous cell in sweep order
    F prev_a = F(0), prev_b = F(0);  // forward: lx, ly of that cell; factor: ax, ay
    // FP32 form, forward solve: this lane's sum of q*q over its cells (sigma,
    // see pcg_job), fused FP32 products over one staged block of diagonals,
    // then added in FP64 (keeps the FP64 pipe, 1/64 of the FP32 rate on this
    // part, off the per-cell path).
    constexpr bool kQQ = KIND == 1 && sizeof(F) == 4;
    double qq = 0.0;

    // Halo prefetch: lane l < kHB holds the word of the column that the
    // waiting lane reaches at step t0 + l, and where needed the lower
    // neighbour's coefficients.
    unsigned long long hpre = kSentinel;
    F spre_a = F(0), spre_b = F(0);
    auto halo_col = [&](int t) { return bwd ? D - 32 - t : t; };
    auto prefetch = [&](int t0) {
        if constexpr (IN) {
            const int xc = halo_col(t0 + lane);
            const bool need = lane < kHB && xc >= 0 && xc < W;
            hpre = hload_if(in, xc, need, kSentinel);
            if constexpr (KIND == 0) {
                if (need) {
                    const size_t k = sd.slot(xc, s * 32 - 1);
                    spre_a = axp[k];
                    spre_b = ayp[k];
                }
            } else if constexpr (KIND == 1 && !kPair) {
                if (need) {
                    F a, b, c, d;
                    ld4(micp + 4 * sd.slot(xc, s * 32 - 1), a, b, c, d);
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
        ring_wait(R, A.fl);
        const char *sbuf = g_smem + R.buf + st * Ring<F>::kStageBytes;
        const F *g0 = (const F *)sbuf;
        const F *g1 = (const F *)(sbuf + S1);
        const F *g2 = (const F *)(sbuf + 2 * S1);
        const uint8_t *gnb = (const uint8_t *)(sbuf + 3 * S1);
        float qq32 = 0.f;
        for (int sub = 0; sub < kB / kHB; sub++) {
            const int t0 = blk * kB + sub * kHB;
            // stage this sub-block's operands in registers
            F o0[kHB], o1[kHB], o2[kHB], o3[kHB];
            unsigned ob[kHB];
#pragma unroll
            for (int jj = 0; jj < kHB; jj++) {
                const int j = sub * kHB + jj;
                const int e = (bwd ? (kB - 1 - j) : j) * 32 + lane;  // slot inside the staged block
                if constexpr (KIND == 0) {
                    o0[jj] = g0[e];
                    o1[jj] = g1[e];
                    o2[jj] = g2[e];
                    ob[jj] = gnb[e];
                    o3[jj] = F(0);
                } else {
                    F w3;
                    o0[jj] = g0[e];
                    ld4(g2 + 4 * e, o1[jj], o2[jj], o3[jj], w3);
                    ob[jj] = nb_of(w3);
                }
            }
            // this sub-block's halo words, then the next sub-block's prefetch
            unsigned long long hw = 0ull;
            F ha = F(0), hb = F(0);
            if constexpr (IN) {
                const int xc = halo_col(t0 + lane);
                const bool need = lane < kHB && xc >= 0 && xc < W;
                hw = halo_take_warp(in, xc, need, hpre, A.fl);
                if (!need) hw = 0ull;
                ha = spre_a;
                hb = spre_b;
                prefetch(t0 + kHB);
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
                    if constexpr (IN) {
                        const double hpc = hdec<double>(__shfl_sync(FULL, hw, jj));
                        const F hax = __shfl_sync(FULL, ha, jj), hay = __shfl_sync(FULL, hb, jj);
                        if (lane == 0) {
                            pc_d = hpc;
                            ax_d = hax;
                            ay_d = hay;
                        }
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
                    F q_d = __shfl_up_sync(FULL, prev, 1);
                    F ly_d = __shfl_up_sync(FULL, prev_b, 1);
                    if constexpr (IN) {
                        F hq, hly;
                        if constexpr (kPair) {
                            const unsigned long long wj = __shfl_sync(FULL, hw, jj);
                            hq = __uint_as_float((unsigned)wj);
                            hly = __uint_as_float((unsigned)(wj >> 32));
                        } else {
                            hq = hdec<F>(__shfl_sync(FULL, hw, jj));
                            hly = __shfl_sync(FULL, hb, jj);
                        }
                        if (lane == 0) {
                            q_d = hq;
                            ly_d = hly;
                        }
                    }
                    F tt = o0[jj];
                    tt = (b & NB_LEFT) ? msub(tt, prev_a, prev) : tt;
                    tt = (b & NB_DOWN) ? msub(tt, ly_d, q_d) : tt;
                    val = tt * o3[jj];
                    prev_a = o1[jj];
                    prev_b = o2[jj];
                } else {
                    // backward substitution (3-conjugate-gradients/Fluid.cpp:289-303)
                    F z_u = __shfl_down_sync(FULL, prev, 1);
                    if constexpr (IN) {
                        const F hz = hdec<F>(__shfl_sync(FULL, hw, jj));
                        if (lane == 31) z_u = hz;
                    }
                    F tt = o0[jj];
                    tt = (b & NB_RIGHT) ? msub(tt, o1[jj], prev) : tt;
                    tt = (b & NB_UP) ? msub(tt, o2[jj], z_u) : tt;
                    val = tt * o3[jj];
                }
                res[jj] = val;
                prev = val;
                // hand the boundary value on at once (one predicated store)
                {
                    const int t = t0 + jj;
                    const int x = (bwd ? D - 1 - t : t) - lane;
                    unsigned long long wv;
                    if constexpr (kPair)
                        wv = (unsigned long long)__float_as_uint(val) | ((unsigned long long)__float_as_uint(o2[jj]) << 32);
                    else
                        wv = henc(val);
                    hstore_if(out, x, wv, producer && rowok && x >= 0 && x < W);
                }
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
                        if (self) pcp[i] = pcv;
                        st4(micp + 4 * i, self ? (F)((double)o1[jj] * pcv) : F(0),
                            self ? (F)((double)o2[jj] * pcv) : F(0), self ? (F)pcv : F(0), nb_word(b, F(0)));
                    } else {
                        if (b & NB_SELF) {
                            zout[i] = res[jj];
                            if constexpr (kQQ) qq32 = fmaf((float)res[jj], (float)res[jj], qq32);
                        }
                    }
                }
            }
        }
        if constexpr (kQQ) qq += (double)qq32;
    }
    if constexpr (kQQ) {
        // the strip's partial: lanes by a fixed shuffle tree (independent of
        // which warp of which team sweeps the strip)
        qq = warp_sum(qq);
        if (lane == 0) A.partials[2 * (size_t)((sd.S * D + kChunk - 1) / kChunk) + s] = qq;
    }
    __syncwarp();
}

template <int KIND, typename F>
__device__ __forceinline__ void sweep_strip_any(const PcgArgs<F> &A, int s, Ring<F> &R, const Chan in,
                                                const Chan out) {
    if (in.valid) sweep_strip<KIND, F, true>(A, s, R, in, out);
    else sweep_strip<KIND, F, false>(A, s, R, in, out);
}

// Sweep of all strips of this block.  The team's T.size*K sweeping warps take
// the strips round-robin: warp `base` sweeps strips base, base + P, base + 2P,
// ... (P = T.size*K), in increasing order for the factor and the forward
// solve and in decreasing order for the backward solve, so that every strip
// waits only on a strip that is swept earlier by its own warp or by another
// warp in the same or an earlier round (no cycle).  A team therefore needs
// fewer blocks than its scene has strips: while a tall scene's pipeline fills
// and drains, the warps that would idle in a one-strip-per-warp schedule sweep
// their next strip.  When every warp has a single strip, the halo rows between
// the warps of one block live in shared memory; otherwise every strip hands its
// boundary row over through its own global row (a shared row would be reused
// by the next round while its reader may still need it).
// hsm_off: byte offset in g_smem of the K-1 shared halo rows (D words each).
template <int KIND, typename F>
__device__ void sweep(const PcgArgs<F> &A, const Team &T, Ring<F> &R, unsigned hsm_off, int nstrips_blk) {
    const int w = threadIdx.x >> 5;
    if (w >= nstrips_blk) return;
    const SDIdx sd = A.sd;
    const int P = T.size * A.K;
    const int base = T.rank * A.K + w;
    const size_t D = sd.D;
    unsigned long long *up = A.halo, *down = A.halo + (size_t)sd.S * D;
    auto smem_row = [&](int k) {
        return Chan{(unsigned long long *)(g_smem + hsm_off + 8u * (unsigned)(k * D)), true};
    };
    auto glob_row = [&](unsigned long long *row) { return Chan{row, true}; };
    const bool one_round = sd.S <= P;
    const int nmine = (sd.S - base + P - 1) / P;  // strips of this warp
    for (int j0 = 0; j0 < nmine; j0++) {
        const int s = base + (KIND == 2 ? nmine - 1 - j0 : j0) * P;
        Chan in{nullptr, false}, out{nullptr, false};
        if (KIND != 2) {  // rows travel upward: strip s takes from s-1, gives to s+1
            if (s > 0) in = (one_round && w > 0) ? smem_row(w - 1) : glob_row(up + (size_t)(s - 1) * D);
            if (s + 1 < sd.S)
                out = (one_round && w + 1 < nstrips_blk) ? smem_row(w) : glob_row(up + (size_t)s * D);
        } else {          // downward: strip s takes from s+1, gives to s-1
            if (s + 1 < sd.S)
                in = (one_round && w + 1 < nstrips_blk) ? smem_row(w) : glob_row(down + (size_t)(s + 1) * D);
            if (s > 0) out = (one_round && w > 0) ? smem_row(w - 1) : glob_row(down + (size_t)s * D);
        }
        sweep_strip_any<KIND, F>(A, s, R, in, out);
    }
}

// Shared-memory layout of a PCG block: ring mbarriers (32 bytes per sweeping
// warp) | staging mbarriers (8 bytes per warp, kMaxWarps) | the K-1 halo rows
// between its strips (D words each) | the per-warp rings.
constexpr unsigned kStageBars = 8u * kMaxWarps;
__host__ __device__ __forceinline__ unsigned halo_offset(int K) { return 32u * K + kStageBars; }
__host__ __device__ __forceinline__ unsigned ring_offset(int K, int D) {
    const size_t nh = (size_t)(K > 1 ? K - 1 : 0) * D;
    return (unsigned)(((halo_offset(K) + nh * 8 + 127) / 128) * 128);
}

// Per-warp ring and staging state; the mbarriers are initialised once per launch.
template <typename F>
__device__ void ring_init(Ring<F> &R, int K, int stages) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    R.bars = 32u * warp;
    R.stages = stages;
    R.ii = R.ci = 0;
    R.dead = false;
    R.sbar = 32u * K + 8u * warp;
    R.sphase = 0;
    R.sdead = false;
    if (lane == 0) {
        if (warp < K)
            for (int k = 0; k < stages; k++) mbar_init(R.bar(k), 1);
        mbar_init(R.stage_bar(), 1);
        fence_mbar_init();
    }
}

// ------------------------------------------------ staged elementwise passes
// The elementwise passes stream their operands through shared memory: for each
// unit of U consecutive diagonals (U a power of two dividing the 16-diagonal
// reduction chunk) lane 0 issues one bulk copy per array (completion on the
// warp's staging mbarrier), so that the warp has its whole unit (6-12 KB) in
// flight at once, not the few loads its registers hold; the lanes then compute
// from shared memory.  Per-cell arithmetic and each lane's accumulation order
// are those of a direct pass over the same cells.
__device__ __forceinline__ void fence_proxy_async_shared() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// Largest unit (rows of 32 slots) whose staged bytes fit the warp's area.
__device__ __forceinline__ int unit_rows(unsigned area, unsigned bytes_per_row) {
    int U = kChunk;
    while (U > 1 && (unsigned)U * bytes_per_row > area) U >>= 1;
    return U;
}
// Wait for the unit in flight.  Like the ring, a timeout elsewhere does not
// shorten it (the copies complete); a copy that never completes marks the
// staging area dead, after which the warp issues and waits for nothing more.
template <typename F>
__device__ __forceinline__ void stage_wait(Ring<F> &R, const Flags &flags) {
    long long n = 0;
    while (!R.sdead && !mbar_try_wait(R.stage_bar(), R.sphase & 1u)) {
        if (++n > kMbarWaitLimit) {
            set_timeout(flags);
            R.sdead = true;
        }
    }
    R.sdead = __any_sync(FULL, R.sdead);
    R.sphase++;
}
// Rows [lo, hi) of a strip-diagonal array (clipped to [0, rows)) into shared
// memory at dst, where row `base` lands at slot 0; returns the bytes copied.
template <typename T>
__device__ __forceinline__ unsigned stage_rows(unsigned dst, const T *src, int base, int lo, int hi, int rows,
                                               uint64_t *bar) {
    lo = lo < 0 ? 0 : lo;
    hi = hi > rows ? rows : hi;
    if (hi <= lo) return 0u;
    const unsigned bytes = (unsigned)(hi - lo) * 32u * sizeof(T);
    bulk_g2s(g_smem + dst + (unsigned)(lo - base) * 32u * sizeof(T), src + (size_t)lo * 32, bytes, bar);
    return bytes;
}
template <typename T>
__device__ __forceinline__ unsigned clipped_bytes(int lo, int hi, int rows) {
    lo = lo < 0 ? 0 : lo;
    hi = hi > rows ? rows : hi;
    return hi > lo ? (unsigned)(hi - lo) * 32u * sizeof(T) : 0u;
}

// One complete solve (factor and/or PCG, by A.mode) of one scene by team T.
// The shared halo rows must hold the sentinel on entry; they hold it again on
// exit (every word a strip hands on is taken by its neighbour).
template <typename F, int kThreads>
__device__ void pcg_job(const PcgArgs<F> &A, const Team &T, Ring<F> &R, double *sm) {
    constexpr int kWarps = kThreads / 32;
    const SDIdx sd = A.sd;
    const int W = sd.W, H = sd.H, D = sd.D;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rows = sd.S * D;  // diagonals of all strips
    const int gwarp = T.rank * kWarps + warp, nwarps = T.size * kWarps;
    // Elementwise phases work on chunks of kChunk diagonals; each warp takes a
    // contiguous run of chunks (the neighbouring diagonals a cell reads are then
    // mostly its own: L1 hits).  Every reduction is summed per chunk (lanes in
    // diagonal order, then a fixed shuffle tree) and the chunk partials in
    // chunk order, so the result depends on the scene alone, not on the number
    // of blocks or warps that solve it: a scene gives bit-identical results in
    // a single-scene launch, in any batch and with any launch shape.
    const int nchunk = (rows + kChunk - 1) / kChunk;
    const int c_per = (nchunk + nwarps - 1) / nwarps;
    const int c_begin = min(nchunk, gwarp * c_per), c_end = min(nchunk, c_begin + c_per);
    auto chunk_put = [&](int slot, int c, double v, bool is_max) {
        v = is_max ? warp_max(v) : warp_sum(v);
        if (lane == 0) A.partials[(size_t)slot * nchunk + c] = v;
    };
    // Lane l adds the partials of chunks l, l+32, l+64, ... in that order; the
    // loads (from L2: other blocks wrote them before the team barrier) are
    // issued eight at a time, so a scene of thousands of chunks costs a few
    // memory latencies, not one per 32 chunks.
    // n: the slot's number of partials (chunks; strips for sigma).
    auto chunk_total = [&](int slot, bool is_max, int n) -> double {
        if (threadIdx.x < 32) {
            double acc = 0.0;
            const double *pt = A.partials + (size_t)slot * nchunk;
            for (int c0 = lane; c0 < n; c0 += 32 * 8) {
                double v[8];
#pragma unroll
                for (int j = 0; j < 8; j++) v[j] = c0 + 32 * j < n ? __ldcg(pt + c0 + 32 * j) : 0.0;
#pragma unroll
                for (int j = 0; j < 8; j++)
                    if (c0 + 32 * j < n) acc = is_max ? smax(acc, v[j]) : acc + v[j];
            }
            acc = is_max ? warp_max(acc) : warp_sum(acc);
            if (lane == 0) sm[kMaxWarps] = acc;
        }
        __syncthreads();
        const double r = sm[kMaxWarps];
        __syncthreads();
        return r;
    };
    // sweeping warps of this block that own at least one strip
    int nstrips_blk = sd.S - T.rank * A.K;
    nstrips_blk = nstrips_blk < 0 ? 0 : (nstrips_blk > A.K ? A.K : nstrips_blk);
    constexpr bool kF32 = !std::is_same<F, double>::value;
    const unsigned hsm_off = halo_offset(A.K);
    R.buf = ring_offset(A.K, D) + (unsigned)warp * A.stages * Ring<F>::kStageBytes;

    // Staging area of this warp: its share of the block's ring memory.
    R.sbytes = (A.K * A.stages * Ring<F>::kStageBytes / kWarps) & ~127u;
    R.sbuf = ring_offset(A.K, D) + (unsigned)warp * R.sbytes;
    // Lane 0 of a warp starts a unit's copies: the warp's reads of the previous
    // unit are done (syncwarp), then a proxy fence orders them before the
    // asynchronous writes into the same shared memory.
    auto unit_begin = [&]() -> bool {
        __syncwarp();
        if (lane != 0 || R.sdead) return false;
        fence_proxy_async_shared();
        return true;
    };

    // sigma = z . r over the red cells (3-conjugate-gradients/Fluid.cpp:356, 376).
    // FP64 form: a separate pass after the backward solve, z_i * r_i as the
    // reference forms them (FP64 products on the sweeping warp's chain would
    // cost the wavefront more than the pass).  Staged: z, r and the neighbour
    // bits of a unit.
    auto dot_zr = [&]() {
        constexpr unsigned kRow = 32u * (sizeof(F) + 8 + 1);
        const int U = unit_rows(R.sbytes, kRow);
        const unsigned oz = R.sbuf, orr = oz + U * 32u * sizeof(F), onb = orr + U * 32u * 8u;
        if (lane == 0) fence_proxy_async_global();  // generic-proxy writes of the sweeps -> bulk copies
        for (int c = c_begin; c < c_end; c++) {
            double acc = 0.0;
            for (int r0 = c * kChunk; r0 < (c + 1) * kChunk; r0 += U) {
                if (unit_begin()) {
                    mbar_expect_tx(R.stage_bar(), U * kRow);
                    stage_rows(oz, A.z, r0, r0, r0 + U, rows, R.stage_bar());
                    stage_rows(orr, A.r, r0, r0, r0 + U, rows, R.stage_bar());
                    stage_rows(onb, A.nb, r0, r0, r0 + U, rows, R.stage_bar());
                }
                stage_wait(R, A.fl);
                const F *sz = (const F *)(g_smem + oz);
                const double *sr = (const double *)(g_smem + orr);
                const uint8_t *snb = (const uint8_t *)(g_smem + onb);
                for (int u = 0; u < U; u++) {
                    const int k = u * 32 + lane;
                    if (snb[k] & NB_RED) acc = acc + (double)sz[k] * sr[k];
                }
            }
            chunk_put(2, c, acc, false);
        }
    };
    // FP32 form: sigma is taken as q . q, q = L^-1 r the forward solve's result.
    // The MIC(0) apply is z = L^-T L^-1 r with L's diagonal 1/precon and its
    // strictly lower part aPlus*precon of the column's cell (the forward solve's
    // coefficients; the backward solve uses the same ones transposed, also after
    // FP32 rounding), so z . r = (L^-1 r) . (L^-1 r) exactly, and in floating
    // point within the rounding of the two triangular solves.  The forward sweep
    // adds q*q up per strip (slot 2 holds one partial per strip): no pass over z
    // and r and no team barrier for it.  Cells outside the masked MIC(0) work
    // hold q = 0 (and r = 0: the right-hand side and A*s vanish there), so they
    // add nothing to either form.
    auto sigma_of_sweeps = [&]() -> double {
        if constexpr (kF32) {
            return chunk_total(2, false, sd.S);
        } else {
            dot_zr();
            team_barrier(T, A.fl);
            return chunk_total(2, false, nchunk);
        }
    };

    // s = z + beta*s (first iteration: s = z), then z' = A s and z'.s over a
    // unit of U diagonals of one strip (3-conjugate-gradients/Fluid.cpp:361-362,
    // 375, 315-332).  Staged: z, s, neighbour bits of the diagonals r0-1 ..
    // r0+U (left/down and right/up neighbours inside the strip), aPlusX and
    // aPlusY of r0-1 .. r0+U-1, aDiag of the unit.  The lower neighbour of lane
    // 0 and the upper neighbour of lane 31 live in the adjacent strips; lanes
    // 0..U-1 and 16..16+U-1 load them and hand them over by shuffle.
    // kAllRed (the unmasked pressure solves of steps 3-5, whose every cell is
    // red): the neighbour bits are neither staged nor read, as every in-grid
    // neighbour takes the s-update.
    auto matvec = [&](int iter, double beta, auto all_red_tag) -> void {
        constexpr bool kAllRed = decltype(all_red_tag)::value;
        const F fbeta = (F)beta;
        auto need = [](int v) {
            return (unsigned)(v + 2) * 32u * (2u * sizeof(F) + (kAllRed ? 0u : 1u)) + (unsigned)v * 32u * sizeof(F) +
                   2u * (unsigned)(v + 1) * 32u * sizeof(F);
        };
        int U = kChunk;
        while (U > 1 && need(U) > R.sbytes) U >>= 1;
        const unsigned rz = (unsigned)(U + 2) * 32u * sizeof(F), rn = kAllRed ? 0u : (unsigned)(U + 2) * 32u,
                       ra = (unsigned)U * 32u * sizeof(F), rxy = (unsigned)(U + 1) * 32u * sizeof(F);
        const unsigned oz = R.sbuf, os = oz + rz, onb = os + rz, oad = onb + rn, oax = oad + ra, oay = oax + rxy;
        const F *__restrict__ zp = A.z;
        const F *__restrict__ so = (iter & 1) ? A.sb : A.sa;
        F *__restrict__ sn = (iter & 1) ? A.sa : A.sb;
        double *__restrict__ asp = A.as;
        if (lane == 0) fence_proxy_async_global();
        for (int c = c_begin; c < c_end; c++) {
            double dacc = 0.0;
            const int s = (c * kChunk) / D;  // a chunk lies inside one strip (D is a multiple of it)
            for (int r0 = c * kChunk; r0 < (c + 1) * kChunk; r0 += U) {
                const int d0 = r0 - s * D;
                if (unit_begin()) {
                    uint64_t *bar = R.stage_bar();
                    const unsigned tx = 2u * clipped_bytes<F>(r0 - 1, r0 + U + 1, rows) +
                                        (kAllRed ? 0u : clipped_bytes<uint8_t>(r0 - 1, r0 + U + 1, rows)) +
                                        clipped_bytes<F>(r0, r0 + U, rows) + 2u * clipped_bytes<F>(r0 - 1, r0 + U, rows);
                    mbar_expect_tx(bar, tx);
                    stage_rows(oz, zp, r0 - 1, r0 - 1, r0 + U + 1, rows, bar);
                    stage_rows(os, so, r0 - 1, r0 - 1, r0 + U + 1, rows, bar);
                    if (!kAllRed) stage_rows(onb, A.nb, r0 - 1, r0 - 1, r0 + U + 1, rows, bar);
                    stage_rows(oad, A.adiag, r0, r0, r0 + U, rows, bar);
                    stage_rows(oax, A.ax, r0 - 1, r0 - 1, r0 + U, rows, bar);
                    stage_rows(oay, A.ay, r0 - 1, r0 - 1, r0 + U, rows, bar);
                }
                // neighbours in the adjacent strips (loaded while the copies fly)
                F xz = F(0), xs = F(0), xa = F(0);
                unsigned xn = 0u;
                {
                    const int j = lane & 15, d = d0 + j;
                    if (j < U && lane < 16 && s > 0 && d < W && 32 * s < H) {  // below lane 0 of diagonal d
                        const size_t k = sd.slot(d, 32 * s - 1);
                        xz = zp[k];
                        xs = so[k];
                        if (!kAllRed) xn = A.nb[k];
                        xa = A.ay[k];
                    } else if (j < U && lane >= 16 && d - 31 >= 0 && d - 31 < W && 32 * s + 32 < H) {  // above lane 31
                        const size_t k = sd.slot(d - 31, 32 * s + 32);
                        xz = zp[k];
                        xs = so[k];
                        if (!kAllRed) xn = A.nb[k];
                    }
                }
                stage_wait(R, A.fl);
                const F *szv = (const F *)(g_smem + oz);
                const F *ssv = (const F *)(g_smem + os);
                const uint8_t *snb = (const uint8_t *)(g_smem + onb);
                const F *sad = (const F *)(g_smem + oad);
                const F *sax = (const F *)(g_smem + oax);
                const F *say = (const F *)(g_smem + oay);
                // A register window slides along the unit's diagonals: row r0+u-1
                // (L: the left neighbour), r0+u (C: the cell) and r0+u+1 (R: the
                // right neighbour) of this lane; the lower neighbour is lane-1's L
                // and the upper one lane+1's R (shuffles), lanes 0 and 31 take
                // theirs from the adjacent strips.  Per diagonal a lane loads only
                // row R and the cell's coefficients.  A neighbour outside the grid
                // holds whatever its slot holds and is not used (fl).
                F zL = szv[lane], sL = ssv[lane], zC = szv[32 + lane], sC = ssv[32 + lane];
                F axL = sax[lane], ayL = say[lane];
                unsigned nL = 0u, nC = 0u;
                if constexpr (!kAllRed) {
                    nL = snb[lane];
                    nC = snb[32 + lane];
                }
                for (int u = 0; u < U; u++) {
                    const F dz = __shfl_sync(FULL, xz, u), ds = __shfl_sync(FULL, xs, u), da = __shfl_sync(FULL, xa, u);
                    const unsigned dn = kAllRed ? 0u : __shfl_sync(FULL, xn, u);
                    const F uz = __shfl_sync(FULL, xz, 16 + u), us = __shfl_sync(FULL, xs, 16 + u);
                    const unsigned un = kAllRed ? 0u : __shfl_sync(FULL, xn, 16 + u);
                    const int x = d0 + u - lane, y = s * 32 + lane;
                    const bool in = x >= 0 && x < W && y < H;
                    const bool hl = in && x > 0, hd = in && y > 0, hr = in && x < W - 1, hu = in && y < H - 1;
                    const int kr = (u + 2) * 32 + lane;
                    const F zR = szv[kr], sR = ssv[kr];
                    const unsigned nR = kAllRed ? (unsigned)NB_RED : (unsigned)snb[kr];
                    F zD = __shfl_up_sync(FULL, zL, 1), sD = __shfl_up_sync(FULL, sL, 1);
                    F aD = __shfl_up_sync(FULL, ayL, 1);
                    F zU = __shfl_down_sync(FULL, zR, 1), sU = __shfl_down_sync(FULL, sR, 1);
                    unsigned nD = kAllRed ? (unsigned)NB_RED : __shfl_up_sync(FULL, nL, 1);
                    unsigned nU = kAllRed ? (unsigned)NB_RED : __shfl_down_sync(FULL, nR, 1);
                    if (lane == 0) {
                        zD = dz;
                        sD = ds;
                        aD = da;
                        if constexpr (!kAllRed) nD = dn;
                    }
                    if (lane == 31) {
                        zU = uz;
                        sU = us;
                        if constexpr (!kAllRed) nU = un;
                    }
                    const F axC = sax[(u + 1) * 32 + lane], ayC = say[(u + 1) * 32 + lane];
                    F vz[5] = {zC, zL, zD, zR, zU}, vs[5] = {sC, sL, sD, sR, sU};
                    // aDiag of the cell, aPlusX of the left neighbour, aPlusY of the
                    // lower one, aPlusX and aPlusY of the cell
                    F va[5] = {sad[u * 32 + lane], axL, hd ? aD : F(0), axC, ayC};
                    unsigned vn[5] = {kAllRed ? (unsigned)NB_RED : nC, kAllRed ? (unsigned)NB_RED : nL, nD, nR, nU};
                    zL = zC;
                    sL = sC;
                    zC = zR;
                    sC = sR;
                    axL = axC;
                    ayL = ayC;
                    if constexpr (!kAllRed) {
                        nL = nC;
                        nC = nR;
                    }
                    const unsigned fl = (in ? 2u : 0u) | (hl ? 4u : 0u) | (hd ? 8u : 0u) | (hr ? 16u : 0u) |
                                        (hu ? 32u : 0u);
                    F sv[5];
#pragma unroll
                    for (int q = 0; q < 5; q++)
                        sv[q] = iter == 0 ? vz[q] : ((vn[q] & NB_RED) ? F(vz[q] + vs[q] * fbeta) : vs[q]);
                    // FP64 form: FP64 accumulation in the reference's order.  FP32
                    // form, pressure matrices (rows sum to zero in the reference:
                    // aDiag = sum of the face factors, each off-diagonal = -factor):
                    // the form sum_j a_ij (s_j - s_i), in FP32 fused multiply-adds.
                    // It keeps the zero row sums exactly (with the FP32-rounded aDiag
                    // the plain form left a tiny, non-zero eigenvalue that made CG
                    // stagnate on some scenes, up to the 2000-iteration cap), and its
                    // terms carry no cancellation between the diagonal and the
                    // neighbours, so FP32 accumulation suffices: against a
                    // float-float sum, the 512-scene batch ran the same iteration
                    // counts (to 3 of 639 on the longest solve) with a pressure error
                    // against the FP64 reference of 1.5e-6 (8e-7), 7 % faster.
                    // Other FP32-form matrices (heat): a float-float sum of the
                    // exact products on the FP32 pipes (GB300 runs FP64 at 1/64 of
                    // the FP32 rate).
                    double t;
                    if constexpr (kF32) {
                        if (A.rowsum_zero) {
                            float tf = 0.f;
#pragma unroll
                            for (int q = 1; q < 5; q++)
                                if (fl & (2u << q)) tf = fmaf(va[q], sv[q] - sv[0], tf);
                            t = (double)tf;
                        } else {
                            FF acc = ff_prod(va[0], sv[0]);
#pragma unroll
                            for (int q = 1; q < 5; q++)
                                if (fl & (2u << q)) acc = ff_add(acc, ff_prod(va[q], sv[q]));
                            t = (double)acc.hi + (double)acc.lo;
                        }
                    } else {
                        t = (double)va[0] * (double)sv[0];
#pragma unroll
                        for (int q = 1; q < 5; q++)
                            t = (fl & (2u << q)) ? t + (double)va[q] * (double)sv[q] : t;
                    }
                    const size_t i = (size_t)(r0 + u) * 32 + lane;
                    sn[i] = in ? sv[0] : F(0);
                    asp[i] = in ? t : 0.0;
                    if (in && (vn[0] & NB_RED))
                        dacc = kF32 ? fma(t, (double)sv[0], dacc) : dacc + t * (double)sv[0];
                }
            }
            chunk_put(1, c, dacc, false);
        }
    };

    // p += alpha s; r -= alpha z'; maxError = |r|_inf  (:363-366), staged
    // p, r, A*s, s and the neighbour bits of a unit.
    // kAllRed: the red cells are the grid's own cells (no neighbour bits staged).
    auto axpy = [&](int iter, double alpha, auto all_red_tag) -> void {
        constexpr bool kAllRed = decltype(all_red_tag)::value;
        constexpr unsigned kRow = 32u * (8u + 8u + 8u + sizeof(F) + (kAllRed ? 0u : 1u));
        const int U = unit_rows(R.sbytes, kRow);
        const unsigned op = R.sbuf, orr = op + U * 256u, oas = orr + U * 256u, osn = oas + U * 256u,
                       onb = osn + U * 32u * sizeof(F);
        const F *__restrict__ snp = (iter & 1) ? A.sa : A.sb;  // the s this iteration's matvec wrote
        double *__restrict__ pp = A.p;
        double *__restrict__ rp = A.r;
        F *rfp = A.rf;  // aliases r in the FP64 form (not written there)
        if (lane == 0) fence_proxy_async_global();
        for (int c = c_begin; c < c_end; c++) {
            unsigned long long mx = 0ull;  // bits of the largest |r| so far
            const int s = (c * kChunk) / D, y = s * 32 + lane;  // the chunk's strip, this lane's row
            for (int r0 = c * kChunk; r0 < (c + 1) * kChunk; r0 += U) {
                if (unit_begin()) {
                    uint64_t *bar = R.stage_bar();
                    mbar_expect_tx(bar, U * kRow);
                    stage_rows(op, A.p, r0, r0, r0 + U, rows, bar);
                    stage_rows(orr, A.r, r0, r0, r0 + U, rows, bar);
                    stage_rows(oas, A.as, r0, r0, r0 + U, rows, bar);
                    stage_rows(osn, snp, r0, r0, r0 + U, rows, bar);
                    if (!kAllRed) stage_rows(onb, A.nb, r0, r0, r0 + U, rows, bar);
                }
                stage_wait(R, A.fl);
                const double *sp = (const double *)(g_smem + op);
                const double *sr = (const double *)(g_smem + orr);
                const double *sas = (const double *)(g_smem + oas);
                const F *ssn = (const F *)(g_smem + osn);
                const uint8_t *snb = (const uint8_t *)(g_smem + onb);
                for (int u = 0; u < U; u++) {
                    const int k = u * 32 + lane;
                    bool red;
                    if constexpr (kAllRed) {
                        const int x = r0 + u - s * D - lane;
                        red = x >= 0 && x < W && y < H;
                    } else {
                        red = snb[k] & NB_RED;
                    }
                    if (red) {
                        const size_t i = (size_t)(r0 + u) * 32 + lane;
                        // FP32 form: one rounding per update (fused); FP64 form: the
                        // reference's two
                        pp[i] = kF32 ? fma((double)ssn[k], alpha, sp[k]) : sp[k] + (double)ssn[k] * alpha;
                        const double rn = kF32 ? fma(sas[k], -alpha, sr[k]) : sr[k] + sas[k] * -alpha;
                        rp[i] = rn;
                        if (kF32) rfp[i] = (F)rn;
                        // std::max(maxError, |r|) on the bit patterns: non-negative
                        // doubles order as unsigned integers; a NaN (above +inf) is
                        // skipped, as (maxError < NaN) is false
                        const unsigned long long b =
                            (unsigned long long)__double_as_longlong(rn) & 0x7fffffffffffffffull;
                        if (b <= 0x7ff0000000000000ull && b > mx) mx = b;
                    }
                }
            }
            chunk_put(0, c, __longlong_as_double((long long)mx), true);
        }
    };

    if (A.mode & PCG_FACTOR) {
        sweep<0, F>(A, T, R, hsm_off, nstrips_blk);
        team_barrier(T, A.fl);
    }
    if (!(A.mode & PCG_SOLVE)) return;

    // p = 0; maxError = |r|_inf   (3-conjugate-gradients/Fluid.cpp:350, 354)
    for (int c = c_begin; c < c_end; c++) {
        double mx = 0.0;
        for (int row = c * kChunk; row < min(rows, (c + 1) * kChunk); row++) {
            const size_t i = (size_t)row * 32 + lane;
            A.p[i] = 0.0;
            if (kF32) A.rf[i] = (F)A.r[i];
            if (A.nb[i] & NB_RED) mx = smax(mx, fabs(A.r[i]));
        }
        chunk_put(0, c, mx, true);
    }
    if (kF32) team_barrier(T, A.fl);  // FP32 copy of r complete
    // z = M^-1 r  (:351)
    sweep<1, F>(A, T, R, hsm_off, nstrips_blk);
    team_barrier(T, A.fl);
    sweep<2, F>(A, T, R, hsm_off, nstrips_blk);
    team_barrier(T, A.fl);

    double maxError = chunk_total(0, true, nchunk);
    double sigma = sigma_of_sweeps();
    int iterations = 0, status;
    if (A.pinned >= 0 ? A.pinned == 0 : maxError < kTol) {
        status = 1;
    } else {
        status = 2;
        double beta = 0.0;
        // the search direction alternates between sa and sb (the matvec reads one
        // and writes the other): iteration k writes sb when k is even
        for (int iter = 0; iter < A.limit; iter++) {
            // block-uniform: every thread of the block leaves together
            if (__syncthreads_or(threadIdx.x == 0 && timed_out(A.fl))) break;
            // s = z + beta*s (first iteration: s = z), then z' = A s and z'.s  (:361-362, 375)
            if (A.all_red) matvec(iter, beta, std::true_type{});
            else matvec(iter, beta, std::false_type{});
            team_barrier(T, A.fl);
            const double alpha = sigma / chunk_total(1, false, nchunk);
            // p += alpha s; r -= alpha z'; maxError = |r|_inf  (:363-366)
            if (A.all_red) axpy(iter, alpha, std::true_type{});
            else axpy(iter, alpha, std::false_type{});
            team_barrier(T, A.fl);
            maxError = chunk_total(0, true, nchunk);
            iterations = iter + 1;
            if (A.pinned >= 0 ? iterations >= A.pinned : maxError < kTol) {
                status = 0;
                break;
            }
            // z = M^-1 r; sigmaNew = z.r  (:372-376)
            sweep<1, F>(A, T, R, hsm_off, nstrips_blk);
            team_barrier(T, A.fl);
            sweep<2, F>(A, T, R, hsm_off, nstrips_blk);
            team_barrier(T, A.fl);
            const double sigmaNew = sigma_of_sweeps();
            beta = sigmaNew / sigma;
            sigma = sigmaNew;
        }
        if (status == 2) iterations = A.limit;
    }
    if (T.rank == 0 && threadIdx.x == 0) {
        A.out->iterations = iterations;
        A.out->status = status;
        A.out->max_error = maxError;
        atomicAdd(A.iter_total, (unsigned long long)iterations);
    }
}

template <typename F, int kThreads>
__global__ void __launch_bounds__(kThreads, 1) pcg_kernel(PcgArgs<F> A) {
    __shared__ double sm[kMaxWarps + 1];
    const Team T{(int)blockIdx.x, (int)gridDim.x, A.barrier, A.partials};
    Ring<F> R;
    ring_init(R, A.K, A.stages);
    const size_t nh = (size_t)(A.K > 1 ? A.K - 1 : 0) * A.sd.D;
    for (size_t k = threadIdx.x; k < nh; k += kThreads)
        ((unsigned long long *)(g_smem + halo_offset(A.K)))[k] = kSentinel;
    __syncthreads();
    pcg_job<F, kThreads>(A, T, R, sm);
}

// ------------------------------------------------------------ batched solves
// Many independent scenes in one cooperative launch.  The grid is cut into
// teams; a team of g blocks solves scenes of up to g*K strips.  Teams of one
// size form a class and take that class's scenes from a shared queue (largest
// estimated work first), so a team that finishes early takes the next scene.
struct BatchTeams {
    const int2 *block_team;   // per block: {team, rank in team}
    const int2 *team;         // per team: {blocks, class}
    const int2 *class_range;  // per class: {offset, count} into class_jobs
    const int *class_jobs;    // job indices, each class in queue order
    int *class_next;          // queue heads (zero at launch)
    int *team_job;            // job taken by each team
    unsigned *team_bar;       // two barrier words per team (zero at launch)
    unsigned *all;            // launch-wide status word
    const int4 *ctl;          // per job: {pinned pressure, pinned heat, limit pressure, limit heat}
    // Placement of teams across SMs: the hardware puts consecutive blocks of a
    // launch on the same few SMs, so a team of consecutive block indices would
    // share those SMs' pipes.  Each block instead takes the slot
    // (its rank on its SM) x nsm + (its SM's dense index), and teams are built
    // from consecutive slots, i.e. from blocks on different SMs.
    const short *sm_dense;    // %smid -> dense SM index (-1: unknown); 1024 entries
    int *sm_fill;             // blocks placed per SM (zero at launch)
    unsigned *grid_bar;       // two barrier words over the whole grid (zero at launch)
    unsigned *remap_fail;     // set when a block could not be placed (zero at launch)
    int nsm, per, remap;
    long long wait_limit;     // polls of one halo or barrier wait
};

// At most 128 registers per thread whatever the block size.
template <typename F, int kThreads>
__global__ void __launch_bounds__(kThreads, 512 / kThreads)
    pcg_batch_kernel(const PcgArgs<F> *jobs, BatchTeams B, int mode, int heat, int pinned, int K, int stages) {
    __shared__ double sm[kMaxWarps + 1];
    __shared__ PcgArgs<F> sA;
    __shared__ int s_slot;
    const Flags launch_fl{B.all, B.all, B.wait_limit};
    if (threadIdx.x == 0) {
        int slot = (int)blockIdx.x;
        if (B.remap) {
            unsigned smid;
            asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
            const int d = smid < 1024u ? B.sm_dense[smid] : -1;
            const int k = d >= 0 ? atomicAdd(B.sm_fill + d, 1) : B.per;
            if (d >= 0 && k < B.per) slot = k * B.nsm + d;
            else atomicOr(B.remap_fail, 1u);
        }
        s_slot = slot;
    }
    if (B.remap) {
        // every block learns whether all of them were placed, then all follow the same rule
        const Team G{(int)blockIdx.x, (int)gridDim.x, B.grid_bar, nullptr};
        team_barrier(G, launch_fl);
        if (threadIdx.x == 0 && ld_volatile(B.remap_fail)) s_slot = (int)blockIdx.x;
    }
    __syncthreads();
    const int2 bt = B.block_team[s_slot];
    const int2 tm = B.team[bt.x];
    Team T{bt.y, tm.x, B.team_bar + 2 * bt.x, nullptr};
    Ring<F> R;
    ring_init(R, K, stages);
    __syncthreads();
    for (;;) {
        if (T.rank == 0 && threadIdx.x == 0) {
            const int2 cr = B.class_range[tm.y];
            const int k = atomicAdd(B.class_next + tm.y, 1);
            *(volatile int *)(B.team_job + bt.x) = k < cr.y ? B.class_jobs[cr.x + k] : -1;
        }
        team_barrier(T, launch_fl);
        const int j = *(volatile int *)(B.team_job + bt.x);
        if (j < 0) break;
        for (int k = threadIdx.x; k < (int)(sizeof(PcgArgs<F>) / 4); k += kThreads)
            ((unsigned *)&sA)[k] = ((const unsigned *)(jobs + j))[k];
        __syncthreads();
        if (threadIdx.x == 0) {
            const int4 c = B.ctl[j];
            sA.mode = mode;
            sA.limit = heat ? c.w : c.z;
            sA.pinned = pinned >= -1 ? pinned : (heat ? c.y : c.x);
            sA.K = K;
            sA.stages = stages;
            sA.fl.all = B.all;
            sA.fl.limit = B.wait_limit;
        }
        // halo rows start at the sentinel: the shared rows of this block
        // (their length changes with the scene) and the scene's global rows
        const size_t nh = (size_t)(K > 1 ? K - 1 : 0) * sA.sd.D;
        for (size_t k = threadIdx.x; k < nh; k += kThreads)
            ((unsigned long long *)(g_smem + halo_offset(K)))[k] = kSentinel;
        const size_t ng = 2 * (size_t)sA.sd.S * sA.sd.D;
        for (size_t k = (size_t)T.rank * kThreads + threadIdx.x; k < ng; k += (size_t)T.size * kThreads)
            sA.halo[k] = kSentinel;
        T.partials = sA.partials;
        team_barrier(T, sA.fl);
        pcg_job<F, kThreads>(sA, T, R, sm);
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
size_t smem_bytes(int K, int D, int stages = kStages) {
    return ring_offset(K, D) + (size_t)K * stages * Ring<F>::kStageBytes;
}

template <typename F, int kThreads>
int max_coresident(size_t smem) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaFuncSetAttribute(pcg_kernel<F, kThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, pcg_kernel<F, kThreads>, kThreads, smem);
    return sms * (per > 2 ? 2 : per);
}

}  // namespace

template <typename F>
int pcg_max_blocks() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return 2 * sms;
}

namespace {
template <typename F>
PcgArgs<F> make_args(const Scene<F> &S, const PcgScratch &X, int heat) {
    PcgArgs<F> A;
    std::memset(&A, 0, sizeof A);
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
    A.fl = Flags{S.flags, S.flags};
    A.out = X.out + (heat ? 1 : 0);
    A.iter_total = X.iter_total;
    A.rowsum_zero = heat ? 0 : 1;
    A.all_red = (!heat && S.variant < 6) ? 1 : 0;
    return A;
}
}  // namespace

namespace {
// FP32-form work arrays of an FP64 scene, and the conversion of its matrix.
PcgArgs<float> make_args_f32(const Scene<double> &S, const PcgF32 &M, const PcgScratch &X, int heat) {
    PcgArgs<float> A;
    std::memset(&A, 0, sizeof A);
    A.sd = S.sd;
    A.adiag = M.adiag;
    A.ax = M.ax;
    A.ay = M.ay;
    A.pc = S.pc;
    A.mic = M.mic;
    A.nb = S.nb;
    A.r = S.r;
    A.p = S.p;
    A.as = S.as;
    A.rf = M.rf;
    A.z = M.z;
    A.sa = M.sa;
    A.sb = M.sb;
    A.partials = X.partials;
    A.barrier = X.barrier;
    A.halo = X.halo;
    A.fl = Flags{S.flags, S.flags};
    A.out = X.out + (heat ? 1 : 0);
    A.iter_total = X.iter_total;
    A.rowsum_zero = heat ? 0 : 1;
    A.all_red = (!heat && S.variant < 6) ? 1 : 0;
    return A;
}
__global__ void matrix_to_f32_kernel(const double *a, const double *b, const double *c, float *fa, float *fb,
                                     float *fc, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        fa[i] = (float)a[i];
        fb[i] = (float)b[i];
        fc[i] = (float)c[i];
    }
}
}  // namespace

template <typename F>
cudaError_t launch_pcg_with(PcgArgs<F> A, const SDIdx &sd, const PcgScratch &X, const PcgConfig &cfg,
                            cudaStream_t st, int *blocks_used);

template <typename F>
cudaError_t launch_pcg(const Scene<F> &S, const PcgScratch &X, const PcgConfig &cfg, cudaStream_t st,
                       int *blocks_used) {
    return launch_pcg_with<F>(make_args(S, X, cfg.heat), S.sd, X, cfg, st, blocks_used);
}

cudaError_t launch_pcg_f32(const Scene<double> &S, const PcgF32 &M, const PcgScratch &X, const PcgConfig &cfg,
                           cudaStream_t st, int *blocks_used) {
    if (cfg.mode & PCG_FACTOR) {  // the FP32 form stores the matrix in FP32 (rounded once)
        const size_t n = S.sd.total();
        matrix_to_f32_kernel<<<(int)std::min<size_t>((n + 255) / 256, 152 * 8), 256, 0, st>>>(
            S.adiag, S.ax, S.ay, M.adiag, M.ax, M.ay, n);
    }
    return launch_pcg_with<float>(make_args_f32(S, M, X, cfg.heat), S.sd, X, cfg, st, blocks_used);
}

template <typename F>
cudaError_t launch_pcg_with(PcgArgs<F> A, const SDIdx &sd, const PcgScratch &X, const PcgConfig &cfg,
                            cudaStream_t st, int *blocks_used) {
    A.mode = cfg.mode;
    A.limit = cfg.limit;
    A.pinned = cfg.pinned;
    A.K = strips_per_block<F>();
    if (A.K > sd.S) A.K = sd.S;
    A.stages = kStages;
    A.fl.limit = cfg.wait_limit > 0 ? cfg.wait_limit : kWaitLimit;
    const size_t smem = smem_bytes<F>(A.K, sd.D);
    const int threads = 512;
    const void *fn = (const void *)pcg_kernel<F, 512>;
    int maxb = max_coresident<F, 512>(smem);
    if (maxb > X.max_blocks) maxb = X.max_blocks;
    const int need = (sd.S + A.K - 1) / A.K;  // blocks that own strips
    if (maxb < need) return cudaErrorInvalidConfiguration;
    // one block per 2048 slots (fewer blocks for small grids measured slower:
    // the elementwise passes lose more than the cheaper barriers save)
    const long long slots = (long long)sd.total();
    int want = (int)((slots + threads * 4 - 1) / (threads * 4));
    if (want < need) want = need;
    int G = want < maxb ? want : maxb;
    if (blocks_used) *blocks_used = G;
    cudaError_t e = cudaMemsetAsync(X.barrier, 0, 2 * sizeof(unsigned), st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(X.halo, 0xff, 2 * (size_t)sd.S * sd.D * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    void *args[] = {&A};
    return cudaLaunchCooperativeKernel(fn, dim3(G), dim3(threads), args, smem, st);
}

// ------------------------------------------------------- batched solves, host
struct PcgBatchPlan {
    int precision = 0;  // sizeof(F)
    int n = 0;
    PcgShape shape{};
    int grid = 0;      // co-resident blocks of the launch
    int max_team = 128;  // largest team the planner may form
    size_t smem = 0;
    std::vector<int> strips, diags, cells;
    // device: [jobs pressure][jobs heat][block_team][team][class_range][class_jobs][team_job]
    //         [zeroed at launch: class_next | team_bar | all]
    char *dev = nullptr;
    size_t dev_bytes = 0;
    void *jobs[2] = {nullptr, nullptr};
    int4 *ctl = nullptr;
    BatchTeams B{};
    size_t tab_off = 0, tab_bytes = 0;  // host-built tables copied each schedule
    size_t zero_off = 0, zero_bytes = 0;
    char *host = nullptr;  // pinned staging of the tables
    cudaEvent_t uploaded = nullptr;
    int nclass = 0;
};

namespace {
constexpr int kMaxClasses = 8;  // team sizes 1, 2, 4, ... 128 blocks; class kMaxClasses: idle blocks
constexpr int kMaxSmid = 1024;

// Which %smid values this device's blocks run on.
__global__ void smid_probe_kernel(int *seen) {
    unsigned smid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    if (threadIdx.x == 0 && smid < (unsigned)kMaxSmid) seen[smid] = 1;
}
size_t al256(size_t v) { return (v + 255) / 256 * 256; }

template <typename F>
const void *batch_fn(int threads) {
    if (threads == 32) return (const void *)pcg_batch_kernel<F, 32>;
    if (threads == 64) return (const void *)pcg_batch_kernel<F, 64>;
    return threads == 128 ? (const void *)pcg_batch_kernel<F, 128> : (const void *)pcg_batch_kernel<F, 256>;
}
}  // namespace

template <typename F>
PcgBatchPlan *pcg_batch_create(const Scene<F> *const *scenes, const PcgScratch *const *scratch, int n,
                               const PcgShape &shape, std::string *err) {
    auto fail = [&](const std::string &m) -> PcgBatchPlan * {
        if (err) *err = m;
        return nullptr;
    };
    if (n <= 0) return fail("empty batch");
    if ((shape.threads != 32 && shape.threads != 64 && shape.threads != 128 && shape.threads != 256) || shape.K < 1 ||
        shape.K > shape.threads / 32 ||
        shape.stages < 2 || shape.stages > 4)
        return fail("unsupported batched PCG shape");
    int dmax = 0;
    for (int i = 0; i < n; i++) dmax = std::max(dmax, scenes[i]->sd.D);
    const size_t smem = smem_bytes<F>(shape.K, dmax, shape.stages);
    const void *fn = batch_fn<F>(shape.threads);
    int dev = 0, sms = 0, per = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    // the attribute stays at the device maximum, so a launch (or a graph
    // replay) of any plan is valid whatever plan was created last
    if (smem + sizeof(PcgArgs<F>) + 1024 > (size_t)optin ||
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - 2048) != cudaSuccess) {
        cudaGetLastError();
        return fail("shared memory per block exceeds the device limit");
    }
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, shape.threads, smem);
    const int grid = sms * per;
    if (grid < 1) return fail("too few co-resident blocks for the batched PCG shape");

    PcgBatchPlan *P = new PcgBatchPlan;
    P->precision = (int)sizeof(F);
    P->n = n;
    P->shape = shape;
    P->grid = grid;
    P->smem = smem;
    for (int i = 0; i < n; i++) {
        P->strips.push_back(scenes[i]->sd.S);
        P->diags.push_back(scenes[i]->sd.D);
        P->cells.push_back(scenes[i]->w * scenes[i]->h);
    }
    size_t off = 0;
    const size_t o_jobs0 = off;
    off = al256(off + n * sizeof(PcgArgs<F>));
    const size_t o_jobs1 = off;
    off = al256(off + n * sizeof(PcgArgs<F>));
    P->tab_off = off;
    const size_t o_bt = off;
    off = al256(off + grid * sizeof(int2));
    const size_t o_team = off;
    off = al256(off + grid * sizeof(int2));
    const size_t o_cr = off;
    off = al256(off + (kMaxClasses + 1) * sizeof(int2));
    const size_t o_cj = off;
    off = al256(off + n * sizeof(int));
    P->tab_bytes = off - P->tab_off;
    const size_t o_ctl = off;
    off = al256(off + n * sizeof(int4));
    const size_t o_tj = off;
    off = al256(off + grid * sizeof(int));
    P->zero_off = off;
    const size_t o_cn = off;
    off += (kMaxClasses + 1) * sizeof(int);
    const size_t o_tb = off;
    off += 2 * grid * sizeof(unsigned);
    const size_t o_all = off;
    off += sizeof(unsigned);
    const size_t o_fill = off;
    off += sms * sizeof(int);
    const size_t o_gbar = off;
    off += 2 * sizeof(unsigned);
    const size_t o_rfail = off;
    off += sizeof(unsigned);
    P->zero_bytes = off - P->zero_off;
    off = al256(off);
    const size_t o_dense = off;
    off += kMaxSmid * sizeof(short);
    P->dev_bytes = al256(off);
    if (cudaMalloc(&P->dev, P->dev_bytes) != cudaSuccess ||
        cudaMallocHost(&P->host, P->tab_bytes) != cudaSuccess ||
        cudaEventCreateWithFlags(&P->uploaded, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        pcg_batch_destroy(P);
        return fail("device allocation for the batched PCG tables failed");
    }
    P->jobs[0] = P->dev + o_jobs0;
    P->jobs[1] = P->dev + o_jobs1;
    P->B.block_team = (const int2 *)(P->dev + o_bt);
    P->B.team = (const int2 *)(P->dev + o_team);
    P->B.class_range = (const int2 *)(P->dev + o_cr);
    P->B.class_jobs = (const int *)(P->dev + o_cj);
    P->B.team_job = (int *)(P->dev + o_tj);
    P->B.class_next = (int *)(P->dev + o_cn);
    P->B.team_bar = (unsigned *)(P->dev + o_tb);
    P->B.all = (unsigned *)(P->dev + o_all);
    P->ctl = (int4 *)(P->dev + o_ctl);
    P->B.ctl = P->ctl;
    P->B.sm_fill = (int *)(P->dev + o_fill);
    P->B.grid_bar = (unsigned *)(P->dev + o_gbar);
    P->B.remap_fail = (unsigned *)(P->dev + o_rfail);
    P->B.sm_dense = (const short *)(P->dev + o_dense);
    P->B.nsm = sms;
    P->B.per = per;
    P->B.remap = 0;
    {
        // dense SM indices from a probe launch with many small blocks
        int *seen = (int *)(P->dev + o_fill);  // scratch before first use
        std::vector<int> hs(kMaxSmid, 0);
        std::vector<short> dense(kMaxSmid, -1);
        int *dseen = nullptr;
        if (cudaMalloc(&dseen, kMaxSmid * sizeof(int)) == cudaSuccess &&
            cudaMemset(dseen, 0, kMaxSmid * sizeof(int)) == cudaSuccess) {
            smid_probe_kernel<<<sms * 16, 32>>>(dseen);
            if (cudaMemcpy(hs.data(), dseen, kMaxSmid * sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess) {
                int n = 0;
                for (int i = 0; i < kMaxSmid; i++)
                    if (hs[i]) dense[i] = (short)n++;
                if (n == sms) P->B.remap = 1;
            }
        }
        cudaGetLastError();
        if (dseen) cudaFree(dseen);
        (void)seen;
        if (cudaMemcpy((void *)P->B.sm_dense, dense.data(), kMaxSmid * sizeof(short), cudaMemcpyHostToDevice) !=
            cudaSuccess) {
            cudaGetLastError();
            P->B.remap = 0;
        }
    }
    std::vector<PcgArgs<F>> a0(n), a1(n);
    for (int i = 0; i < n; i++) {
        a0[i] = make_args(*scenes[i], *scratch[i], 0);
        a1[i] = make_args(*scenes[i], *scratch[i], 1);
    }
    if (cudaMemcpy(P->jobs[0], a0.data(), n * sizeof(PcgArgs<F>), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(P->jobs[1], a1.data(), n * sizeof(PcgArgs<F>), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        pcg_batch_destroy(P);
        return fail("upload of the batched PCG jobs failed");
    }
    return P;
}

void pcg_batch_destroy(PcgBatchPlan *P) {
    if (!P) return;
    if (P->uploaded) {
        cudaEventSynchronize(P->uploaded);
        cudaEventDestroy(P->uploaded);
    }
    if (P->host) cudaFreeHost(P->host);
    if (P->dev) cudaFree(P->dev);
    delete P;
}

int pcg_batch_grid(const PcgBatchPlan *P) { return P->grid; }
size_t pcg_batch_table_bytes(const PcgBatchPlan *P) { return P->tab_bytes; }
void pcg_batch_set_max_team(PcgBatchPlan *P, int blocks) { P->max_team = blocks > 0 ? blocks : 128; }

// Teams and queues from a cost model: work(i, g) = estimated time of scene i's
// solves on a team of g blocks.  Scene i starts in class first_class[i] (teams
// of 2^c blocks).  Every non-empty class gets one team; then, while blocks are
// left, the class with the latest estimated finish (its queue, largest scene
// first, handed to whichever of its teams frees first) gets one more team or
// teams twice as large (up to max_team blocks), whichever shortens that
// finish most per block spent, as long as it improves.  Each queue is ordered by work, largest first.
// teams[c] and tsize[c] give the teams of class c; returns the blocks in
// teams, or -1 when the classes' first teams alone exceed the grid.
int pcg_plan_teams_fn(int grid, int n, const int *first_class, const PlanWork &work, int *teams, int *tsize,
                      std::vector<std::vector<int>> *queues, int max_team) {
    std::vector<std::vector<int>> members(kMaxClasses);
    for (int i = 0; i < n; i++) {
        const int c = first_class[i];
        if (c < 0 || c >= kMaxClasses) return -1;
        members[c].push_back(i);
    }
    int size[kMaxClasses];
    // Finish time of a class: its queue (largest first) served by `nt` teams of
    // g blocks, each job taken by the team that frees first.
    std::vector<double> loads;  // min-heap of the teams' busy times
    auto finish = [&](int c, int nt, int g) {
        loads.assign(std::min<size_t>(nt, members[c].size()), 0.0);
        double fin = 0.0;
        for (int i : members[c]) {
            std::pop_heap(loads.begin(), loads.end(), std::greater<double>());
            loads.back() += work(i, g);
            fin = std::max(fin, loads.back());
            std::push_heap(loads.begin(), loads.end(), std::greater<double>());
        }
        return fin;
    };
    double fin[kMaxClasses];
    for (int c = 0; c < kMaxClasses; c++) {
        size[c] = 1 << c;
        std::stable_sort(members[c].begin(), members[c].end(),
                         [&](int a, int b) { return work(a, 1 << c) > work(b, 1 << c); });
    }
    int left = grid;
    for (int c = 0; c < kMaxClasses; c++) {
        teams[c] = members[c].empty() ? 0 : 1;
        left -= teams[c] << c;
        fin[c] = members[c].empty() ? 0.0 : finish(c, 1, size[c]);
    }
    if (left < 0) return -1;
    for (;;) {
        int best = -1;
        double bt = -1.0;
        for (int c = 0; c < kMaxClasses; c++) {
            if (!members[c].empty() && fin[c] > bt) {
                bt = fin[c];
                best = c;
            }
        }
        if (best < 0) break;
        const int c = best, sz = size[c];
        // more teams of the current size: the fewest that shorten the finish
        // (with jobs of equal size one more team may not)
        int add = 0;
        double fin_add = bt;
        for (int k = 1; teams[c] + k <= (int)members[c].size() && k * sz <= left; k++) {
            fin_add = finish(c, teams[c] + k, sz);
            if (fin_add < bt) {
                add = k;
                break;
            }
        }
        const bool can_add = add > 0;
        // every team of the class twice as large
        const bool can_grow = sz * 2 <= max_team && teams[c] * sz <= left;
        const double fin_grow = can_grow ? finish(c, teams[c], 2 * sz) : bt;
        // the option that shortens the finish most per block spent
        const double gain_add = can_add ? (bt - fin_add) / ((double)add * sz) : 0.0;
        const double gain_grow = can_grow ? (bt - fin_grow) / ((double)teams[c] * sz) : 0.0;
        if (gain_add > 0.0 && gain_add >= gain_grow) {
            teams[c] += add;
            left -= add * sz;
            fin[c] = fin_add;
        } else if (gain_grow > 0.0) {
            left -= teams[c] * sz;
            size[c] = 2 * sz;
            fin[c] = fin_grow;
        } else {
            break;
        }
    }
    for (int c = 0; c < kMaxClasses; c++) tsize[c] = size[c];
    if (queues) *queues = std::move(members);
    return grid - left;
}

// Host preview and the original model: scenes go to the class of the
// smallest power-of-two team that covers their strips (one sweeping warp per
// strip); work = work_sweep (the wavefront part, which more blocks do not
// shorten) + work_elem (the elementwise part at that smallest team, which
// shrinks with the team).
int pcg_plan_teams(int grid, int K, int n, const int *strips, const double *work_sweep,
                   const double *work_elem, int *teams, int *tsize, std::vector<std::vector<int>> *queues,
                   int max_team) {
    std::vector<int> cls(n);
    for (int i = 0; i < n; i++) {
        const int need = (strips[i] + K - 1) / K;
        int c = 0;
        while ((1 << c) < need) c++;
        if (c >= kMaxClasses) return -1;
        cls[i] = c;
    }
    const PlanWork w = [&](int i, int g) {
        return work_sweep[i] + (work_elem ? work_elem[i] * (double)(1 << cls[i]) / g : 0.0);
    };
    return pcg_plan_teams_fn(grid, n, cls.data(), w, teams, tsize, queues, max_team);
}

int pcg_batch_schedule(PcgBatchPlan *P, const int *first_class, const PlanWork &work, cudaStream_t st) {
    int teams[kMaxClasses], tsize[kMaxClasses];
    std::vector<std::vector<int>> members;
    if (pcg_plan_teams_fn(P->grid, P->n, first_class, work, teams, tsize, &members, P->max_team) < 0) return -1;
    // host tables
    if (cudaEventSynchronize(P->uploaded) != cudaSuccess) return -2;  // staging free again
    char *h = P->host;
    const size_t base = P->tab_off;
    auto at = [&](const void *devp) { return h + ((const char *)devp - (P->dev + base)); };
    int2 *bt = (int2 *)at(P->B.block_team);
    int2 *tm = (int2 *)at(P->B.team);
    int2 *cr = (int2 *)at(P->B.class_range);
    int *cj = (int *)at(P->B.class_jobs);
    int blk = 0, team = 0, pos = 0;
    for (int c = 0; c < kMaxClasses; c++) {
        cr[c] = make_int2(pos, (int)members[c].size());
        for (int i : members[c]) cj[pos++] = i;
        for (int t = 0; t < teams[c]; t++, team++) {
            tm[team] = make_int2(tsize[c], c);
            for (int r = 0; r < tsize[c]; r++) bt[blk++] = make_int2(team, r);
        }
    }
    // blocks left over form one-block teams of the empty idle class
    cr[kMaxClasses] = make_int2(pos, 0);
    for (; blk < P->grid; blk++, team++) {
        tm[team] = make_int2(1, kMaxClasses);
        bt[blk] = make_int2(team, 0);
    }
    if (cudaMemcpyAsync(P->dev + base, h, P->tab_bytes, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaEventRecord(P->uploaded, st) != cudaSuccess)
        return -2;
    return 0;
}

int4 *pcg_batch_ctl(PcgBatchPlan *P) { return P->ctl; }

// cfg.pinned >= -1 applies to every scene; -2 takes each scene's entry of the
// control table (cfg.limit is unused: limits come from the table).
template <typename F>
cudaError_t launch_pcg_batch(PcgBatchPlan *P, const PcgConfig &cfg, cudaStream_t st) {
    if (P->precision != (int)sizeof(F)) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(P->dev + P->zero_off, 0, P->zero_bytes, st);
    if (e != cudaSuccess) return e;
    const PcgArgs<F> *jobs = (const PcgArgs<F> *)P->jobs[cfg.heat ? 1 : 0];
    BatchTeams B = P->B;
    B.wait_limit = cfg.wait_limit > 0 ? cfg.wait_limit : kWaitLimit;
    int mode = cfg.mode, heat = cfg.heat, pinned = cfg.pinned, K = P->shape.K, stages = P->shape.stages;
    void *args[] = {&jobs, &B, &mode, &heat, &pinned, &K, &stages};
    return cudaLaunchCooperativeKernel(batch_fn<F>(P->shape.threads), dim3(P->grid), dim3(P->shape.threads), args,
                                       P->smem, st);
}

template PcgBatchPlan *pcg_batch_create<double>(const Scene<double> *const *, const PcgScratch *const *, int,
                                                const PcgShape &, std::string *);
template PcgBatchPlan *pcg_batch_create<float>(const Scene<float> *const *, const PcgScratch *const *, int,
                                               const PcgShape &, std::string *);
template cudaError_t launch_pcg_batch<double>(PcgBatchPlan *, const PcgConfig &, cudaStream_t);
template cudaError_t launch_pcg_batch<float>(PcgBatchPlan *, const PcgConfig &, cudaStream_t);

template cudaError_t launch_pcg<double>(const Scene<double> &, const PcgScratch &, const PcgConfig &,
                                        cudaStream_t, int *);
template cudaError_t launch_pcg<float>(const Scene<float> &, const PcgScratch &, const PcgConfig &,
                                       cudaStream_t, int *);
template int pcg_max_blocks<double>();
template int pcg_max_blocks<float>();

}  // namespace ifl
