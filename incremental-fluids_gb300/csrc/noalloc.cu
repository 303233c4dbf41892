// noalloc.cu - pressure solve that allocates nothing (ifl_pcg_solve_noalloc).
//
// For callers that cannot allocate device memory while they run: code that
// executes inside another framework's memory pool or under a strict memory
// budget, real-time loops that must not enter the allocator, and processes
// where cudaMalloc is forbidden after start-up.  The caller passes the
// matrix, right-hand side and solution as device arrays; every intermediate
// array of the solve lives in one file-scope device array of fixed size.
#include <cstring>
#include <mutex>

#include "ifl_device.cuh"
#include "solver.h"

namespace ifl {
namespace {

// Largest supported problem: strips x diagonals of the strip-diagonal layout,
// S*D <= kMaxStripDiagonals, e.g. 256 x 256 cells (8 strips x 288 diagonals).
constexpr size_t kMaxStripDiagonals = 2304;
constexpr size_t kMaxSlots = kMaxStripDiagonals * 32;
constexpr size_t kMaxBlocks = 512;
// FP64 arrays per slot: adiag, ax, ay, pc, r, p, as, z, sa, sb (10) + MIC record (4)
constexpr size_t kScratchBytes = kMaxSlots * (14 * 8 + 1) + 2 * kMaxStripDiagonals * 8 +
                                 4 * kMaxBlocks * 8 + 1024;

// The shared scratch.  Every GPU that loads the library holds it until exit.
static __device__ __align__(256) unsigned char g_pcg_scratch[kScratchBytes];

static_assert(sizeof(PcgOut) == sizeof(ifl_pcg_stats), "stats layout");

// Device address of g_pcg_scratch per device (in host code the symbol itself
// is only a host-side stand-in, not a device address).
std::mutex g_mu;
void *g_addr[64];

int scratch_address(int dev, void **out) {
    if (dev < 0 || dev >= 64) return IFL_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_pcg_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return IFL_ERR_CUDA;
        }
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return IFL_OK;
}

// Row-major inputs -> strip-diagonal arrays, plus the neighbour bits of the
// unmasked (3-conjugate-gradients) system.
__global__ void noalloc_in_kernel(SDIdx sd, const double *adiag, const double *ax, const double *ay,
                                  const double *rhs, double *sd_adiag, double *sd_ax, double *sd_ay,
                                  double *sd_r, uint8_t *nb) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= sd.W || y >= sd.H) return;
    const size_t c = x + (size_t)y * sd.W, k = sd.slot(x, y);
    sd_adiag[k] = adiag[c];
    sd_ax[k] = ax[c];
    sd_ay[k] = ay[c];
    sd_r[k] = rhs[c];
    nb[k] = NB_SELF | NB_RED | (x > 0 ? NB_LEFT : 0) | (y > 0 ? NB_DOWN : 0) | (x < sd.W - 1 ? NB_RIGHT : 0) |
            (y < sd.H - 1 ? NB_UP : 0);
}

// Strip-diagonal solution -> row-major output; a timed-out bounded wait turns
// the reported status into -1.
__global__ void noalloc_out_kernel(SDIdx sd, const double *sd_p, double *p, const unsigned *flags,
                                   ifl_pcg_stats *stats) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x == 0 && y == 0 && (*flags & FLAG_TIMEOUT)) stats->status = -1;
    if (x >= sd.W || y >= sd.H) return;
    p[x + (size_t)y * sd.W] = sd_p[sd.slot(x, y)];
}

template <typename T>
T *take(unsigned char *&cur, size_t count) {
    cur = (unsigned char *)(((uintptr_t)cur + 255) & ~(uintptr_t)255);
    T *p = (T *)cur;
    cur += count * sizeof(T);
    return p;
}

}  // namespace
}  // namespace ifl

extern "C" int ifl_pcg_solve_noalloc(int w, int h, const double *adiag, const double *aplusx,
                                     const double *aplusy, const double *rhs, double *p, int max_iter,
                                     ifl_pcg_stats *stats, void *stream) {
    using namespace ifl;
    if (w < 2 || h < 2 || max_iter < 0 || !adiag || !aplusx || !aplusy || !rhs || !p || !stats)
        return IFL_ERR_ARG;
    const SDIdx sd = SDIdx::make(w, h);
    if ((size_t)sd.S * sd.D > kMaxStripDiagonals) return IFL_ERR_UNSUPPORTED;  // beyond the scratch size
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return IFL_ERR_CUDA;
    void *base = nullptr;
    if (int e = scratch_address(dev, &base)) return e;
    cudaStream_t st = (cudaStream_t)stream;

    const size_t n = sd.total();
    unsigned char *cur = (unsigned char *)base;
    Scene<double> S{};
    S.sd = sd;
    S.variant = IFL_PLAIN;
    S.w = w;
    S.h = h;
    S.adiag = take<double>(cur, n);
    S.ax = take<double>(cur, n);
    S.ay = take<double>(cur, n);
    S.pc = take<double>(cur, n);
    S.mic = take<double>(cur, 4 * n);
    S.r = take<double>(cur, n);
    S.rf = S.r;
    S.p = take<double>(cur, n);
    S.as = take<double>(cur, n);
    S.z = take<double>(cur, n);
    S.sa = take<double>(cur, n);
    S.sb = take<double>(cur, n);
    S.nb = take<uint8_t>(cur, n);
    S.flags = take<unsigned>(cur, 8);
    PcgScratch X{};
    X.halo = take<unsigned long long>(cur, 2 * (size_t)sd.S * sd.D);
    X.partials = take<double>(cur, 4 * pcg_chunks(sd));
    X.barrier = take<unsigned>(cur, 2);
    X.iter_total = take<unsigned long long>(cur, 1);
    X.out = (PcgOut *)stats;  // the solve writes its outcome straight into the caller's struct
    X.max_blocks = (int)kMaxBlocks;
    if ((size_t)(cur - (unsigned char *)base) > kScratchBytes) return IFL_ERR_UNSUPPORTED;

    // The array keeps the previous call's contents: clear what must start at
    // zero (neighbour bits of the padding slots, status word).
    if (cudaMemsetAsync(S.nb, 0, n, st) != cudaSuccess || cudaMemsetAsync(S.flags, 0, 8 * sizeof(unsigned), st) != cudaSuccess)
        return IFL_ERR_CUDA;
    dim3 b(32, 8), g((w + 31) / 32, (h + 7) / 8);
    noalloc_in_kernel<<<g, b, 0, st>>>(sd, adiag, aplusx, aplusy, rhs, S.adiag, S.ax, S.ay, S.r, S.nb);
    PcgConfig cfg{PCG_FACTOR | PCG_SOLVE, max_iter, -1, 0};
    if (launch_pcg<double>(S, X, cfg, st, nullptr) != cudaSuccess) {
        cudaGetLastError();
        return IFL_ERR_CUDA;
    }
    noalloc_out_kernel<<<g, b, 0, st>>>(sd, S.p, p, S.flags, stats);
    return cudaGetLastError() == cudaSuccess ? IFL_OK : IFL_ERR_CUDA;
}
