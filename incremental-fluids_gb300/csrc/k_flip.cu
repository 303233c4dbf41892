// k_flip.cu - step 8 (FLIP) particle kernels (sm_103a, FP64).
//
// ParticleQuantities of 8-flip/Fluid.cpp (692-940) and the FLIP additions to
// FluidQuantity (296-303, 374-389, 663-690), reorganised for the GPU while
// keeping every floating-point result of the reference:
//
//  * particle -> grid (fromParticles): the reference adds each particle's
//    hat-filter weight into four grid nodes, particles in index order.  Here
//    particles are bucketed by base node (atomic ranks, then each bucket
//    sorted by particle index), and one thread per node merges its four
//    buckets in ascending particle order, so every node's sums are the
//    reference's left-to-right sums;
//  * countParticles / pruneParticles: counts by atomics; the prune is a
//    swap-with-last walk whose outcome depends on order, so it is replayed by
//    one thread over the (usually empty) list of particles in overfull cells;
//  * seedParticles / initParticles: the frand() LCG is jumped ahead to each
//    cell's first draw (2 draws per attempt, exclusive scans over cells give
//    the draw offsets and the output slots), so every cell seeds in parallel;
//  * gridToParticles, diff/undiff and advect are per particle / per node.
//
// The particle count and the LCG state live on the device (FlipState::ctl),
// so a whole update is launched without a host round trip.
#include <algorithm>

#include "ifl_device.cuh"

namespace ifl {

namespace {

constexpr int kMaxPerCell = 12;  // _MaxPerCell
constexpr int kMinPerCell = 3;   // _MinPerCell
constexpr int kAvgPerCell = 4;   // _AvgPerCell
constexpr double kFlipAlpha = 0.001;  // _flipAlpha
constexpr unsigned kLcgA = 1103515245u, kLcgC = 12345u;
constexpr int kScanThreads = 1024;

// ------------------------------------------------------------------ frand
// frand() (8-flip/Fluid.cpp:38-46): s <- (a*s + c) mod 2^31; the value is the
// new state's top 23 bits as a fraction in [0, 1).
__device__ __forceinline__ float frand_next(unsigned &s) {
    s = (s * kLcgA + kLcgC) & 0x7FFFFFFFu;
    return (float)(s >> 8) * 0x1p-23f;
}
// State after k further draws: the affine map raised to the k-th power by
// squaring (all arithmetic mod 2^32, reduced to 31 bits at the end).
__device__ __forceinline__ unsigned frand_jump(unsigned s, unsigned long long k) {
    if (k == 0) return s;
    unsigned A = 1u, C = 0u, ma = kLcgA, mc = kLcgC;
    while (k) {
        if (k & 1ull) {
            A = ma * A;
            C = ma * C + mc;
        }
        mc = ma * mc + mc;
        ma = ma * ma;
        k >>= 1;
    }
    return (A * s + C) & 0x7FFFFFFFu;
}
// `x + frand()` of the reference: int + float in float arithmetic.
__device__ __forceinline__ double jitter(int x, float f) { return (double)__fadd_rn((float)x, f); }

// pointInBody (8-flip/Fluid.cpp:724-731), x and y in grid units.
__device__ __forceinline__ bool point_in_body(const Scene<double> &S, double x, double y) {
    for (int b = 0; b < S.nbodies; b++)
        if (body_distance(S.bodies[b], x * S.hx, y * S.hx) < 0.0) return true;
    return false;
}

__device__ __forceinline__ double lerp_q(const Scene<double> &S, int t, double x, double y) {
    const Quant<double> &Q = S.q[t];
    return q_lerp<double>(Q.src, S.P, Q.w, Q.h, Q.ox, Q.oy, x, y);
}

// ------------------------------------------------------------------- scan
// Exclusive scan of n 64-bit values into out[0..n], out[n] = total: tile
// scans, a scan of the tile sums, then the tile offsets.
__device__ __forceinline__ unsigned long long block_exclusive(unsigned long long v, unsigned long long *sw,
                                                              unsigned long long *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned long long incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) sw[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const unsigned long long wv = lane < nw ? sw[lane] : 0ull;
        unsigned long long wi = wv;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        sw[lane] = wi - wv;
        if (lane == 31) *total = wi;
    }
    __syncthreads();
    const unsigned long long r = sw[warp] + incl - v;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kScanThreads)
    scan_tiles_kernel(const unsigned long long *in, unsigned long long *out, unsigned long long *sums, int n) {
    __shared__ unsigned long long sw[32], tot;
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned long long v = i < n ? in[i] : 0ull;
    const unsigned long long ex = block_exclusive(v, sw, &tot);
    if (i < n) out[i] = ex;
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kScanThreads) scan_sums_kernel(unsigned long long *sums, int ntiles) {
    __shared__ unsigned long long sw[32], tot;
    unsigned long long carry = 0;
    for (int base = 0; base < ntiles; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const unsigned long long v = i < ntiles ? sums[i] : 0ull;
        const unsigned long long ex = block_exclusive(v, sw, &tot);
        if (i < ntiles) sums[i] = carry + ex;
        carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) sums[ntiles] = carry;
}

__global__ void __launch_bounds__(kScanThreads)
    scan_add_kernel(unsigned long long *out, const unsigned long long *sums, int n, int ntiles) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += sums[blockIdx.x];
    if (i == 0) out[n] = sums[ntiles];
}

void scan_u64(const unsigned long long *in, unsigned long long *out, unsigned long long *tmp, int n,
              cudaStream_t st) {
    const int ntiles = (n + kScanThreads - 1) / kScanThreads;
    if (ntiles == 0) {
        cudaMemsetAsync(out, 0, sizeof(unsigned long long), st);
        return;
    }
    scan_tiles_kernel<<<ntiles, kScanThreads, 0, st>>>(in, out, tmp, n);
    scan_sums_kernel<<<1, kScanThreads, 0, st>>>(tmp, ntiles);
    scan_add_kernel<<<ntiles, kScanThreads, 0, st>>>(out, tmp, n, ntiles);
}

inline int particle_blocks(int cap) { return std::max(1, std::min((cap + 255) / 256, 152 * 16)); }
inline int blocks_for(long n, int t) { return (int)std::max(1L, (n + t - 1) / t); }

// ------------------------------------------------------------------- init
// initParticles (8-flip/Fluid.cpp:733-750): 4 jittered attempts per cell in
// row-major order, 2 draws each, attempts inside a body are dropped.
__global__ void init_count_kernel(Scene<double> S, FlipState X) {
    const int n = S.w * S.h;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const int x = c % S.w, y = c / S.w;
    unsigned s = frand_jump((unsigned)X.ctl[FC_RNG], 2ull * kAvgPerCell * c);
    int k = 0;
    for (int i = 0; i < kAvgPerCell; i++) {
        const double px = jitter(x, frand_next(s));
        const double py = jitter(y, frand_next(s));
        k += !point_in_body(S, px, py);
    }
    X.seedv[c] = (unsigned long long)k;
}

__global__ void init_write_kernel(Scene<double> S, FlipState X) {
    const int n = S.w * S.h;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const int x = c % S.w, y = c / S.w;
    unsigned s = frand_jump((unsigned)X.ctl[FC_RNG], 2ull * kAvgPerCell * c);
    long j = (long)X.seedx[c];
    for (int i = 0; i < kAvgPerCell; i++) {
        const double px = jitter(x, frand_next(s));
        const double py = jitter(y, frand_next(s));
        if (point_in_body(S, px, py)) continue;
        X.px[j] = px;
        X.py[j] = py;
        j++;
    }
}

__global__ void init_done_kernel(Scene<double> S, FlipState X) {
    const int n = S.w * S.h;
    X.ctl[FC_COUNT] = (int)X.seedx[n];
    X.ctl[FC_RNG] = (int)frand_jump((unsigned)X.ctl[FC_RNG], 2ull * kAvgPerCell * n);
}

// ------------------------------------------------------ particle -> grid
struct KindGeo {
    int w, h, off;
    double ox, oy;
};
__device__ __forceinline__ KindGeo kind_geo(const Scene<double> &S, const FlipState &X, int k) {
    KindGeo g;
    g.w = k == 1 ? S.w + 1 : S.w;
    g.h = k == 2 ? S.h + 1 : S.h;
    g.off = X.node_off[k];
    g.ox = k == 1 ? 0.0 : 0.5;
    g.oy = k == 2 ? 0.0 : 0.5;
    return g;
}
// fromParticles' clamped sample position relative to the grid
// (8-flip/Fluid.cpp:669-673): max(0.5, min(w - 1.5, p - o)).
__device__ __forceinline__ double clamp_sample(double p, double o, int n) {
    return smax(0.5, smin(n - 1.5, p - o));
}

__global__ void p2g_bucket_kernel(Scene<double> S, FlipState X) {
    const int N = X.ctl[FC_COUNT];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const double px = X.px[i], py = X.py[i];
        for (int k = 0; k < 3; k++) {
            const KindGeo g = kind_geo(S, X, k);
            const int bx = (int)clamp_sample(px, g.ox, g.w), by = (int)clamp_sample(py, g.oy, g.h);
            const int key = g.off + bx + by * g.w;
            X.brank[(long)k * X.cap + i] = (int)atomicAdd(&X.bcount[key], 1ull);
        }
    }
}

__global__ void p2g_scatter_kernel(Scene<double> S, FlipState X) {
    const int N = X.ctl[FC_COUNT];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const double px = X.px[i], py = X.py[i];
        for (int k = 0; k < 3; k++) {
            const KindGeo g = kind_geo(S, X, k);
            const int bx = (int)clamp_sample(px, g.ox, g.w), by = (int)clamp_sample(py, g.oy, g.h);
            const int key = g.off + bx + by * g.w;
            X.blist[X.bstart[key] + X.brank[(long)k * X.cap + i]] = i;
        }
    }
}

// Buckets hold a few particles each: insertion sort by particle index.
__global__ void p2g_sort_kernel(FlipState X) {
    const int key = blockIdx.x * blockDim.x + threadIdx.x;
    if (key >= X.node_off[3]) return;
    int *b = X.blist + X.bstart[key];
    const int n = (int)(X.bstart[key + 1] - X.bstart[key]);
    for (int i = 1; i < n; i++) {
        const int v = b[i];
        int j = i - 1;
        while (j >= 0 && b[j] > v) {
            b[j + 1] = b[j];
            j--;
        }
        b[j + 1] = v;
    }
}

// One thread per node of one kind: the sums of addSample over the particles
// of the (up to) four base buckets around the node, in particle order; then
// the division by the weight, or CELL_EMPTY for a fluid node without weight.
__global__ void p2g_gather_kernel(Scene<double> S, FlipState X) {
    const int k = blockIdx.y;
    const KindGeo g = kind_geo(S, X, k);
    const int node = blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= g.w * g.h) return;
    const int nx = node % g.w, ny = node / g.w;
    long beg[4], end[4];
    int nb = 0;
    for (int by = ny - 1; by <= ny; by++)
        for (int bx = nx - 1; bx <= nx; bx++) {
            if (bx < 0 || by < 0 || bx > g.w - 2 || by > g.h - 2) continue;
            const int key = g.off + bx + by * g.w;
            beg[nb] = (long)X.bstart[key];
            end[nb] = (long)X.bstart[key + 1];
            nb++;
        }
    const int q0 = k == 0 ? 0 : k + 1;  // kind 0: d (and T), 1: u, 2: v
    const double *v0 = X.prop[q0], *v1 = X.prop[1];
    double wsum = 0.0, acc0 = 0.0, acc1 = 0.0;
    for (;;) {
        int best = -1, bi = 0x7fffffff;
        for (int j = 0; j < nb; j++)
            if (beg[j] < end[j] && X.blist[beg[j]] < bi) {
                bi = X.blist[beg[j]];
                best = j;
            }
        if (best < 0) break;
        beg[best]++;
        const double x = clamp_sample(X.px[bi], g.ox, g.w), y = clamp_sample(X.py[bi], g.oy, g.h);
        const double kk = (1.0 - fabs(nx - x)) * (1.0 - fabs(ny - y));
        wsum += kk;
        acc0 += kk * v0[bi];
        if (k == 0) acc1 += kk * v1[bi];
    }
    const long idx = nx + (long)ny * S.P;
    for (int r = 0; r < (k == 0 ? 2 : 1); r++) {
        const int q = r == 0 ? q0 : 1;
        const Quant<double> &Q = S.q[q];
        const double acc = r == 0 ? acc0 : acc1;
        if (wsum != 0.0) {
            Q.src[idx] = acc / wsum;
        } else {
            Q.src[idx] = acc;
            if (Q.cell[idx] == CELL_FLUID) {
                Q.cell[idx] = CELL_EMPTY;
                atomicAdd(&X.ctl[FC_EMPTY + q], 1);
            }
        }
    }
}

// ------------------------------------------------- count / prune / seed
__global__ void count_kernel(Scene<double> S, FlipState X) {
    const int N = X.ctl[FC_COUNT];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const int ix = (int)X.px[i], iy = (int)X.py[i];
        if (ix >= 0 && iy >= 0 && ix < S.w && iy < S.h) atomicAdd(&X.cell_count[ix + iy * S.w], 1);
    }
}

__device__ __forceinline__ void move_particle(const FlipState &X, int dst, int src) {
    X.px[dst] = X.px[src];
    X.py[dst] = X.py[src];
    for (int t = 0; t < 4; t++) X.prop[t][dst] = X.prop[t][src];
}

// pruneParticles (8-flip/Fluid.cpp:767-789): one CTA.  Nothing happens
// unless a cell holds more than 12 particles; then the particles in such
// cells are listed in index order and one thread replays the reference's
// walk (a removed particle is replaced by the last one, which is examined
// next; particles of other cells are never removed).
__global__ void __launch_bounds__(1024) prune_kernel(Scene<double> S, FlipState X) {
    const int w = S.w, h = S.h, ncell = w * h;
    const int N = X.ctl[FC_COUNT];
    int any = 0;
    for (int c = threadIdx.x; c < ncell; c += blockDim.x) any |= X.cell_count[c] > kMaxPerCell;
    if (!__syncthreads_or(any)) return;
    __shared__ int s_warp[32], s_base, s_total;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) s_base = 0;
    __syncthreads();
    for (int base = 0; base < N; base += blockDim.x) {
        const int i = base + threadIdx.x;
        bool f = false;
        if (i < N) {
            const int ix = (int)X.px[i], iy = (int)X.py[i];
            f = ix >= 0 && iy >= 0 && ix < w && iy < h && X.cell_count[ix + iy * w] > kMaxPerCell;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, f);
        if (lane == 0) s_warp[warp] = __popc(bal);
        __syncthreads();
        if (warp == 0) {
            const int v = lane < nw ? s_warp[lane] : 0;
            int incl = v;
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            s_warp[lane] = incl - v;
            if (lane == 31) s_total = incl;
        }
        __syncthreads();
        if (f) X.cand[s_base + s_warp[warp] + __popc(bal & ((1u << lane) - 1u))] = i;
        __syncthreads();
        if (threadIdx.x == 0) s_base += s_total;
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    int cnt = N;
    for (int ci = 0; ci < s_base; ci++) {
        const int p = X.cand[ci];
        if (p >= cnt) break;
        for (;;) {
            const int ix = (int)X.px[p], iy = (int)X.py[p];
            if (ix < 0 || iy < 0 || ix >= w || iy >= h) break;
            const int cell = ix + iy * w;
            if (X.cell_count[cell] <= kMaxPerCell) break;
            move_particle(X, p, --cnt);
            X.cell_count[cell]--;
            if (p >= cnt) break;
        }
        if (p >= cnt) break;
    }
    X.ctl[FC_COUNT] = cnt;
}

// seedParticles (8-flip/Fluid.cpp:791-818): a cell with k < 3 particles makes
// 3 - k attempts of 2 draws each; an attempt is kept unless particle number
// `cell index` (the reference tests that one, not the new particle) is inside
// a body.  Seeding stops once the particle cap is reached.
__global__ void seed_count_kernel(Scene<double> S, FlipState X) {
    const int n = S.w * S.h;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const int att = max(0, kMinPerCell - X.cell_count[c]);
    unsigned long long acc = 0;
    if (att > 0) {
        const int N0 = X.ctl[FC_COUNT];
        if (c >= N0) atomicOr(S.flags, FLAG_FLIP_SEED);  // outside the supported envelope
        else if (!point_in_body(S, X.px[c], X.py[c])) acc = (unsigned long long)att;
    }
    X.seedv[c] = (unsigned long long)att | (acc << 32);
}

__global__ void seed_write_kernel(Scene<double> S, FlipState X) {
    const int n = S.w * S.h;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const unsigned long long v = X.seedv[c];
    const int att = (int)(v & 0xffffffffull);
    if (att == 0) return;
    const bool acc = (v >> 32) != 0;
    const long N0 = X.ctl[FC_COUNT];
    const long room = X.cap - N0;
    const unsigned long long ax = X.seedx[c];
    const long A = (long)(ax & 0xffffffffull), B = (long)(ax >> 32);
    const unsigned s0 = (unsigned)X.ctl[FC_RNG];
    const int x = c % S.w, y = c / S.w;
    for (int i = 0; i < att; i++) {
        const long before = B + (acc ? i : 0);  // accepted attempts ahead of this one
        if (before >= room) return;            // the cap was reached: this attempt never runs
        if (!acc) continue;
        unsigned s = frand_jump(s0, 2ull * (unsigned long long)(A + i));
        const double px = jitter(x, frand_next(s));
        const double py = jitter(y, frand_next(s));
        const long j = N0 + before;
        X.px[j] = px;
        X.py[j] = py;
        for (int t = 0; t < 4; t++) X.prop[t][j] = lerp_q(S, t, px, py);
        if (before == room - 1) X.ctl[FC_EXEC] = (int)(A + i + 1);
    }
}

__global__ void seed_done_kernel(Scene<double> S, FlipState X) {
    const int n = S.w * S.h;
    const unsigned long long tot = X.seedx[n];
    const long att = (long)(tot & 0xffffffffull), acc = (long)(tot >> 32);
    const long N0 = X.ctl[FC_COUNT], room = X.cap - N0;
    long exec = att, N = N0 + acc;
    if (acc >= room) {
        exec = X.ctl[FC_EXEC];
        N = X.cap;
    }
    X.ctl[FC_COUNT] = (int)N;
    X.ctl[FC_RNG] = (int)frand_jump((unsigned)X.ctl[FC_RNG], 2ull * (unsigned long long)exec);
}

// ------------------------------------------------------- grid -> particle
// copy(): _old = _src for every quantity (8-flip/Fluid.cpp:374-376).
__global__ void copy_kernel(Scene<double> S) {
    const Quant<double> &Q = S.q[blockIdx.z];
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= Q.w || y >= Q.h) return;
    const long idx = x + (long)y * S.P;
    Q.dst[idx] = Q.src[idx];
}

// gridToParticles(alpha) (8-flip/Fluid.cpp:886-897) over the diff()ed grid
// (src - (1 - alpha)*old, 8-flip/Fluid.cpp:378-382), formed per sample.
__device__ __forceinline__ double lerp_diff(const Scene<double> &S, int t, double keep, double x, double y) {
    const Quant<double> &Q = S.q[t];
    x = smin(smax(x - Q.ox, 0.0), Q.w - 1.001);
    y = smin(smax(y - Q.oy, 0.0), Q.h - 1.001);
    const int ix = (int)x, iy = (int)y;
    x -= ix;
    y -= iy;
    const long i0 = ix + (long)iy * S.P, i1 = i0 + S.P;
    const double x00 = Q.src[i0] - keep * Q.dst[i0], x10 = Q.src[i0 + 1] - keep * Q.dst[i0 + 1];
    const double x01 = Q.src[i1] - keep * Q.dst[i1], x11 = Q.src[i1 + 1] - keep * Q.dst[i1 + 1];
    return lerp1(lerp1(x00, x10, x), lerp1(x01, x11, x), y);
}

__global__ void g2p_kernel(Scene<double> S, FlipState X, double alpha, int diff) {
    const int N = X.ctl[FC_COUNT];
    const double keep = 1.0 - alpha;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const double x = X.px[i], y = X.py[i];
        for (int t = 0; t < 4; t++) {
            const double l = diff ? lerp_diff(S, t, keep, x, y) : lerp_q(S, t, x, y);
            double p = X.prop[t][i];
            p *= keep;
            p += l;
            X.prop[t][i] = p;
        }
    }
}

// undiff(alpha) after diff(alpha): src = (src - keep*old) + keep*old
// (8-flip/Fluid.cpp:378-389; not the identity in floating point).
__global__ void undiff_kernel(Scene<double> S) {
    const Quant<double> &Q = S.q[blockIdx.z];
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= Q.w || y >= Q.h) return;
    const long idx = x + (long)y * S.P;
    const double keep = 1.0 - kFlipAlpha;
    const double d = Q.src[idx] - keep * Q.dst[idx];
    Q.src[idx] = d + keep * Q.dst[idx];
}

// ParticleQuantities::advect: forward rungeKutta3 (the last stage is not
// divided by hx, as in the reference), backProject, clamp to the domain
// (8-flip/Fluid.cpp:820-870, 916-924).
__global__ void advect_kernel(Scene<double> S, FlipState X, double dt) {
    const int N = X.ctl[FC_COUNT];
    const double hx = S.hx;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        double x = X.px[i], y = X.py[i];
        const double firstU = lerp_q(S, 2, x, y) / hx;
        const double firstV = lerp_q(S, 3, x, y) / hx;
        const double midX = x + 0.5 * dt * firstU;
        const double midY = y + 0.5 * dt * firstV;
        const double midU = lerp_q(S, 2, midX, midY) / hx;
        const double midV = lerp_q(S, 3, midX, midY) / hx;
        const double lastX = x + 0.75 * dt * midU;
        const double lastY = y + 0.75 * dt * midV;
        const double lastU = lerp_q(S, 2, lastX, lastY);
        const double lastV = lerp_q(S, 3, lastX, lastY);
        x += dt * ((2.0 / 9.0) * firstU + (3.0 / 9.0) * midU + (4.0 / 9.0) * lastU);
        y += dt * ((2.0 / 9.0) * firstV + (3.0 / 9.0) * midV + (4.0 / 9.0) * lastV);
        double d = 1e30;
        int nearest = -1;
        for (int b = 0; b < S.nbodies; b++) {
            const double db = body_distance(S.bodies[b], x * hx, y * hx);
            if (db < d) {
                d = db;
                nearest = b;
            }
        }
        if (d < -1.0) {
            x *= hx;
            y *= hx;
            body_closest(S.bodies[nearest], x, y);
            double nx, ny;
            body_normal(S.bodies[nearest], nx, ny, x, y);
            x -= nx * hx;
            y -= ny * hx;
            x /= hx;
            y /= hx;
        }
        X.px[i] = smax(smin(x, S.w - 0.001), 0.0);
        X.py[i] = smax(smin(y, S.h - 0.001), 0.0);
    }
}

inline dim3 quant_grid(const Scene<double> &S, dim3 b) {
    return dim3((S.w + 1 + b.x - 1) / b.x, (S.h + 1 + b.y - 1) / b.y, 4);
}

}  // namespace

// -------------------------------------------------------------- launchers
void launch_flip_init(const Scene<double> &S, const FlipState &X, cudaStream_t st) {
    const int n = S.w * S.h;
    init_count_kernel<<<blocks_for(n, 256), 256, 0, st>>>(S, X);
    scan_u64(X.seedv, X.seedx, X.scan_tmp, n, st);
    init_write_kernel<<<blocks_for(n, 256), 256, 0, st>>>(S, X);
    init_done_kernel<<<1, 1, 0, st>>>(S, X);
    g2p_kernel<<<particle_blocks(X.cap), 256, 0, st>>>(S, X, 1.0, 0);  // gridToParticles(1.0)
}

// particlesToGrid (8-flip/Fluid.cpp:899-912): transfer and extrapolate every
// quantity, then count, prune and seed.
void launch_flip_p2g(const Scene<double> &S, const FlipState &X, cudaStream_t st) {
    const int nodes = X.node_off[3], n = S.w * S.h;
    const int pb = particle_blocks(X.cap);
    cudaMemsetAsync(X.bcount, 0, sizeof(unsigned long long) * nodes, st);
    cudaMemsetAsync(X.ctl + FC_EMPTY, 0, 4 * sizeof(int), st);
    p2g_bucket_kernel<<<pb, 256, 0, st>>>(S, X);
    scan_u64(X.bcount, X.bstart, X.scan_tmp, nodes, st);
    p2g_scatter_kernel<<<pb, 256, 0, st>>>(S, X);
    p2g_sort_kernel<<<blocks_for(nodes, 256), 256, 0, st>>>(X);
    const int gmax = (S.w + 1) * (S.h + 1);
    p2g_gather_kernel<<<dim3(blocks_for(gmax, 256), 3), 256, 0, st>>>(S, X);
    launch_extrapolate_guarded(S, 0xFu, X.ctl + FC_EMPTY, st);
    cudaMemsetAsync(X.cell_count, 0, sizeof(int) * n, st);
    count_kernel<<<pb, 256, 0, st>>>(S, X);
    prune_kernel<<<1, 1024, 0, st>>>(S, X);
    cudaMemsetAsync(X.ctl + FC_EXEC, 0, sizeof(int), st);
    seed_count_kernel<<<blocks_for(n, 256), 256, 0, st>>>(S, X);
    scan_u64(X.seedv, X.seedx, X.scan_tmp, n, st);
    seed_write_kernel<<<blocks_for(n, 256), 256, 0, st>>>(S, X);
    seed_done_kernel<<<1, 1, 0, st>>>(S, X);
}

void launch_flip_copy(const Scene<double> &S, cudaStream_t st) {
    dim3 b(32, 8);
    copy_kernel<<<quant_grid(S, b), b, 0, st>>>(S);
}

// diff, gridToParticles(alpha), undiff (8-flip/Fluid.cpp:1394-1409)
void launch_flip_g2p(const Scene<double> &S, const FlipState &X, cudaStream_t st) {
    g2p_kernel<<<particle_blocks(X.cap), 256, 0, st>>>(S, X, kFlipAlpha, 1);
    dim3 b(32, 8);
    undiff_kernel<<<quant_grid(S, b), b, 0, st>>>(S);
}

void launch_flip_advect(const Scene<double> &S, const FlipState &X, double dt, cudaStream_t st) {
    advect_kernel<<<particle_blocks(X.cap), 256, 0, st>>>(S, X, dt);
}

}  // namespace ifl
