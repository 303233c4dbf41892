// ifl_internal.h - device data layout and kernel launchers of the GB300 solver.
//
// HBM layout of one scene (w x h pressure cells):
//   every 2-D array is row-major with one shared row pitch P (elements),
//   P = round_up(w + 2, 32), and h + 2 rows, so that the largest grid of the
//   scene (the (w+2) x (h+1) / (w+1) x (h+2) corner grids of the distance
//   field) fits, every row starts 128-byte aligned for both element sizes and a
//   cell (x, y) of any grid lives at x + y*P.
// Field storage type F is double (IFL_FP64) or float (IFL_FP32); solid
// geometry (distance, normals, volumes) and the MIC(0) factor stay FP64.
//
// The pressure system (matrix, MIC(0) operands, PCG vectors) uses the
// strip-diagonal layout SDIdx: rows are grouped in 32-row strips and, inside a
// strip, cells are ordered by anti-diagonal d = x + lane (lane = y mod 32),
// 32 lanes contiguous.  A MIC(0) wavefront step of a strip touches exactly one
// diagonal, so every array is read and written as one contiguous 32-element
// line per step and a run of steps is one contiguous block (streamed into
// shared memory by bulk copies).
#pragma once
#include <cstddef>
#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace ifl {

enum : uint8_t { CELL_FLUID = 0, CELL_SOLID = 1, CELL_EMPTY = 2 };

// Neighbour bits consumed by the PCG kernel (one byte per cell).
enum : uint8_t {
    NB_SELF = 1,   // cell takes part in masked MIC(0) work (fluid, or unmasked variant)
    NB_LEFT = 2,   // x-1 term present in MIC(0) factor / forward solve
    NB_DOWN = 4,   // y-1 term present
    NB_RIGHT = 8,  // x+1 term present in backward solve
    NB_UP = 16,    // y+1 term present
    NB_RED = 32    // cell takes part in dot products / max-norm / AXPY
};

// Rigid body with host-computed trigonometry (cos/sin of +theta and -theta are
// evaluated once per update by the host C library, exactly the values the
// reference's rotate() obtains on every call).
struct DevBody {
    int type;  // 0 box, 1 sphere
    int pad_;
    double px, py, sx, sy, vx, vy, vth;
    double cpos, spos, cneg, sneg;
};

// Strip-diagonal index: slot(x, y) = ((s*D + x + l)*32 + l), s = y/32, l = y%32.
// D (diagonals per strip) covers W + 31 and is padded to a multiple of kSweepBlock.
constexpr int kSweepBlock = 16;
struct SDIdx {
    int W, H, S, D;
    __host__ __device__ __forceinline__ size_t slot(int x, int y) const {
        const int s = y >> 5, l = y & 31;
        return ((size_t)s * D + x + l) * 32 + l;
    }
    __host__ __device__ __forceinline__ size_t total() const { return (size_t)S * D * 32; }
    static SDIdx make(int w, int h) {
        SDIdx r;
        r.W = w;
        r.H = h;
        r.S = (h + 31) / 32;
        r.D = (w + 31 + kSweepBlock - 1) / kSweepBlock * kSweepBlock;
        return r;
    }
};

template <typename F>
struct Quant {
    F *src, *dst;
    double *phi, *vol, *nx, *ny;
    uint8_t *cell, *body, *ready;
    int *list;  // extrapolation work lists (2 x P*(h+2) ints)
    int w, h;
    double ox, oy;
};

template <typename F>
struct Scene {
    int variant, w, h, P;
    int nq;  // 3 or 4 quantities
    double hx;
    double rho_air, rho_soot, diffusion, t_amb, g;
    Quant<F> q[4];  // d, t, u, v
    SDIdx sd;          // layout of the pressure-system arrays below
    double *r, *p;     // residual and solution stay FP64 in both forms
    double *as;        // A*s, accumulated in FP64 (a consistent operator in both forms)
    F *rf;             // r in storage precision for the substitutions (aliases r for FP64)
    F *z, *sa, *sb;
    F *adiag, *ax, *ay;
    F *mic;            // MIC(0) apply record per slot: {lx, ly, pc, neighbour bits}
    double *pc;        // MIC(0) factor, FP64
    uint8_t *nb;
    F *udens, *vdens;
    const DevBody *bodies;
    int nbodies;
    unsigned *flags;  // device status word
};

struct PcgOut {
    int iterations;
    int status;
    double max_error;
};

// Diagonals per reduction chunk of the PCG's elementwise phases.
constexpr int kPcgChunk = 16;
inline size_t pcg_chunks(const SDIdx &sd) { return ((size_t)sd.S * sd.D + kPcgChunk - 1) / kPcgChunk; }

// Scratch for the persistent PCG kernel.
struct PcgScratch {
    double *partials;    // 4 reduction slots x pcg_chunks(sd)
    unsigned *barrier;   // 2 words
    unsigned long long *halo;  // 2 x S x D boundary rows handed between strips (sentinel protocol)
    PcgOut *out;
    unsigned long long *iter_total;  // PCG iterations summed over launches
    int max_blocks;
};

enum { PCG_FACTOR = 1, PCG_SOLVE = 2 };

struct PcgConfig {
    int mode;
    int limit;
    int pinned;
    int heat;  // 1: writes to the heat PcgOut slot
    long long wait_limit = 0;  // polls of one device-side wait before it gives up; 0: about a second
};

// Launch shape of the batched PCG kernel (chosen by the batch autotuner).
struct PcgShape {
    int threads;  // 32, 64, 128 or 256 threads per block
    int K;        // strips (sweeping warps) per block, <= threads / 32
    int stages;   // bulk-copy ring stages per sweeping warp, 2..4
};

// Launchers (stream-ordered, no host synchronisation).
template <typename F> void launch_inflow(const Scene<F> &S, int qi, double x0, double y0, double x1,
                                         double y1, double val, cudaStream_t st);
template <typename F> void launch_fill_solid(const Scene<F> &S, cudaStream_t st);
template <typename F> void launch_bc(const Scene<F> &S, cudaStream_t st);
template <typename F> void launch_buoyancy(const Scene<F> &S, double dt, cudaStream_t st);
template <typename F> void launch_assemble(const Scene<F> &S, double dt, int what, cudaStream_t st);
template <typename F> void launch_heat_assemble(const Scene<F> &S, double dt, cudaStream_t st);
template <typename F> void launch_apply_pressure(const Scene<F> &S, double dt, cudaStream_t st);
template <typename F> void launch_extrapolate(const Scene<F> &S, unsigned qmask, cudaStream_t st);
template <typename F> void launch_advect(const Scene<F> &S, double dt, cudaStream_t st);
// strip-diagonal FP64 array -> row-major field (T = p after the heat solve)
template <typename F> void launch_sd_to_rows(const Scene<F> &S, F *rows, const double *sd_arr, cudaStream_t st);
// toImage: 8-bit RGBA of the density (and, heat != 0, the temperature) into a device buffer
template <typename F> void launch_render(const Scene<F> &S, unsigned char *rgba, int heat, cudaStream_t st);
template <typename F> cudaError_t launch_pcg(const Scene<F> &S, const PcgScratch &X, const PcgConfig &c,
                                             cudaStream_t st, int *blocks_used);
template <typename F> int pcg_max_blocks();
// FP32-form solves of an FP64 scene (step 8 with IFL_FP32): FP32 matrix,
// MIC(0) apply records and PCG vectors beside the scene's FP64 r, p, A*s and
// factor; the matrix is rounded from the scene's FP64 one at each factor.
struct PcgF32 {
    float *adiag, *ax, *ay, *mic, *rf, *z, *sa, *sb;
};
cudaError_t launch_pcg_f32(const Scene<double> &S, const PcgF32 &M, const PcgScratch &X, const PcgConfig &c,
                           cudaStream_t st, int *blocks_used);
// Gauss-Seidel solve of steps 1-2 (k_gs.cu): one CTA, h <= gs_max_rows().
template <typename F>
cudaError_t launch_gs(const Scene<F> &S, const PcgScratch &X, double dt, int limit, int pinned, cudaStream_t st,
                      long long wait_limit = 0);
int gs_max_rows();

// Batched PCG: many scenes in one cooperative launch (k_pcg.cu).  The plan
// holds the per-scene job tables and the team/queue tables on the device.
struct PcgBatchPlan;
template <typename F>
PcgBatchPlan *pcg_batch_create(const Scene<F> *const *scenes, const PcgScratch *const *scratch, int n,
                               const PcgShape &shape, std::string *err);
void pcg_batch_destroy(PcgBatchPlan *P);
int pcg_batch_grid(const PcgBatchPlan *P);
size_t pcg_batch_table_bytes(const PcgBatchPlan *P);  // team/queue tables uploaded per schedule
// Estimated time of scene i's solves on a team of g blocks (planner cost model).
using PlanWork = std::function<double(int i, int g)>;
// Rebuilds teams and queues (stream-ordered upload): scene i starts in class
// first_class[i] (teams of 2^c blocks; a team sweeps its scene's strips
// round-robin, so any team size serves any scene).
int pcg_batch_schedule(PcgBatchPlan *P, const int *first_class, const PlanWork &work, cudaStream_t st);
// Team plan (host only): class c holds the scenes that start in it; teams[c]
// teams of tsize[c] blocks serve it; queues[c] = its scenes by decreasing
// work.  Teams grow up to max_team blocks.  Returns the blocks used, -1 if
// the grid is too small.
int pcg_plan_teams_fn(int grid, int n, const int *first_class, const PlanWork &work, int *teams, int *tsize,
                      std::vector<std::vector<int>> *queues, int max_team = 128);
// The same with scenes in the class of the smallest team that gives each of
// their strips its own sweeping warp, work = work_sweep + work_elem scaled by
// the team size (work_elem may be null).
int pcg_plan_teams(int grid, int K, int n, const int *strips, const double *work_sweep,
                   const double *work_elem, int *teams, int *tsize, std::vector<std::vector<int>> *queues,
                   int max_team = 128);
void pcg_batch_set_max_team(PcgBatchPlan *P, int blocks);
// Device table of per-scene {pinned pressure, pinned heat, limit pressure, limit heat}.
int4 *pcg_batch_ctl(PcgBatchPlan *P);
template <typename F> cudaError_t launch_pcg_batch(PcgBatchPlan *P, const PcgConfig &cfg, cudaStream_t st);

// ------------------------------------------------------------ batches
// One inflow rectangle of one quantity (FluidQuantity::addInflow arguments).
struct BatchInflow {
    int q, pad_;
    double x0, y0, x1, y1, val;
};

// Tiles of 32x8 threads that cover every grid of a w x h scene.
inline int batch_tiles(int w, int h, int tw = 32, int th = 8) {
    return ((w + 2 + tw - 1) / tw) * ((h + 2 + th - 1) / th);
}
// Candidate tile shapes (threads x rows) of the batched tiled phases; the
// first is the default.
constexpr int kTileShapes = 6;
constexpr int kTileW[kTileShapes] = {32, 32, 64, 16, 128, 64};
constexpr int kTileH[kTileShapes] = {8, 4, 4, 16, 2, 2};

// Device view of a batch of scenes for the batched phase launches.
template <typename F>
struct SceneBatch {
    const Scene<F> *scenes;        // n scenes
    const int *tile_start;         // n + 1 prefix sums of batch_tiles for tiles of tw x th
    const BatchInflow *inflows;    // inflows of all scenes, scene by scene
    const int *inflow_start;       // n + 1 prefix sums
    int n, tiles;
    int tw, th;                    // tile shape (threads x rows of one block)
};

template <typename F> void launch_batch_inflow(const SceneBatch<F> &B, cudaStream_t st);
template <typename F> void launch_batch_fill_solid(const SceneBatch<F> &B, int variant, int nq, cudaStream_t st);
template <typename F> void launch_batch_bc(const SceneBatch<F> &B, cudaStream_t st);
template <typename F> void launch_batch_buoyancy(const SceneBatch<F> &B, double dt, cudaStream_t st);
template <typename F> void launch_batch_assemble(const SceneBatch<F> &B, double dt, int what, cudaStream_t st);
template <typename F> void launch_batch_heat_assemble(const SceneBatch<F> &B, double dt, cudaStream_t st);
template <typename F> void launch_batch_heat_to_rows(const SceneBatch<F> &B, cudaStream_t st);
template <typename F> void launch_batch_apply_pressure(const SceneBatch<F> &B, double dt, cudaStream_t st);
template <typename F> void launch_batch_extrapolate(const SceneBatch<F> &B, unsigned qmask, cudaStream_t st);
template <typename F> void launch_batch_advect(const SceneBatch<F> &B, double dt, cudaStream_t st);

// ------------------------------------------------------------ step 8: FLIP
// Particle state (FP64 structure of arrays, capacity 12 particles per cell,
// the reference's _maxParticles) and the work tables of its transfers.
// The particle-to-grid transfer runs on three grids: kind 0 = w x h (density
// and temperature share positions and weights), 1 = (w+1) x h (u), 2 =
// w x (h+1) (v); their nodes are numbered densely, kind after kind.
enum FlipCtl {
    FC_COUNT = 0,   // live particles
    FC_RNG = 1,     // frand() LCG state (bits of a uint32)
    FC_EMPTY = 2,   // 2..5: CELL_EMPTY cells of quantity d, T, u, v after the transfer
    FC_EXEC = 6,    // seeding attempts executed when the particle cap was reached
    FC_N0 = 7,      // particles before seeding
    FC_WORDS = 16
};
struct FlipState {
    double *px, *py;
    double *prop[4];                    // d, T, u, v carried by the particles
    int cap;                            // 12 * w * h
    int node_off[4];                    // first node of each kind, node_off[3] = total
    unsigned long long *bcount;         // per node: particles whose base cell is the node
    unsigned long long *bstart;         // exclusive scan of bcount (node_off[3] + 1)
    int *brank;                         // 3 x cap: rank of a particle inside its bucket
    int *blist;                         // 3 x cap: particle indices bucket by bucket
    int *cell_count;                    // w * h particles per cell (countParticles)
    unsigned long long *seedv, *seedx;  // w * h (+1): attempts | accepted << 32, and its scan
    unsigned long long *scan_tmp;       // tile sums of the scans
    int *cand;                          // prune candidates (cap)
    int *ctl;                           // FlipCtl words
};
// Tile sums a scan of n values needs.
inline size_t flip_scan_tiles(size_t n) { return (n + 1023) / 1024 + 2; }

// Launchers (FP64 scenes; stream-ordered, no host synchronisation).
void launch_flip_init(const Scene<double> &S, const FlipState &X, cudaStream_t st);
void launch_flip_p2g(const Scene<double> &S, const FlipState &X, cudaStream_t st);
void launch_flip_copy(const Scene<double> &S, cudaStream_t st);
void launch_flip_g2p(const Scene<double> &S, const FlipState &X, cudaStream_t st);
void launch_flip_advect(const Scene<double> &S, const FlipState &X, double dt, cudaStream_t st);
// Extrapolation of the transfer (k_fields.cu): the parallel DAG relaxation
// for quantities without CELL_EMPTY cells, the order-exact LIFO walk for the
// others (skip[q] selects per quantity, read on the device).
void launch_extrapolate_guarded(const Scene<double> &S, unsigned qmask, const int *empty_counts, cudaStream_t st);

// what-bits for launch_assemble
enum { ASM_RHS = 1, ASM_MATRIX = 2, ASM_DENS = 4 };

// Device flag bits (Scene::flags[0]).
enum : unsigned {
    FLAG_TIMEOUT = 1u,
    FLAG_RING_SOLID = 2u,
    FLAG_FLIP_SEED = 4u,   // seeding tested a particle number beyond the live count
    FLAG_FLIP_STACK = 8u   // the empty-cell extrapolation ran out of its work bound
};

}  // namespace ifl
