// batch.cu - many handles stepped together (ifl_batch_*).
//
// One batch step equals one FluidSolver::update per member
// (3-conjugate-gradients/Fluid.cpp:433-447 ... 7-variable-density/Fluid.cpp:995-1034):
// every phase runs for all members in one launch over a table of their scenes,
// and each PCG solve (heat, pressure) of all members runs in one persistent
// cooperative launch (k_pcg.cu, pcg_batch_kernel).  The launch sequence of a
// step is captured once as a CUDA graph and replayed; per step the host only
// uploads the scene table (source/destination pointers alternate), the body
// tables and the PCG queues, which it reorders by each scene's iteration count
// of the previous step.  The PCG launch shape is chosen by timing candidate
// shapes on the first step's real system (pinned iteration count).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "solver.h"

namespace ifl {

namespace {

__global__ void gather_stats_kernel(PcgOut *const *outs, unsigned *const *flags, PcgOut *dst, unsigned *dflags,
                                    int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dst[2 * i] = outs[i][0];
    dst[2 * i + 1] = outs[i][1];
    dflags[i] = *flags[i];
}

size_t al256(size_t v) { return (v + 255) / 256 * 256; }

constexpr int kMaxBodies = 256;     // per member (ifl_set_bodies limit)
constexpr int kMaxInflowRects = 8;  // per member

int pow2ceil(int v) {
    int p = 1;
    while (p < v) p <<= 1;
    return p;
}

// The home shape (the first candidate) is kept unless another one is more than
// kHomeMargin faster in the trial: a trial of a few pinned iterations of the
// first system cannot separate shapes within a few percent (on GB300 the
// 512-scene batch ran its steps 19 % faster on 64 x 1 x 2 than on 32 x 1 x 2,
// which had won such a trial by 1.4 %).
constexpr double kHomeMargin = 0.05;

template <typename F>
std::vector<PcgShape> candidate_shapes() {
    if (sizeof(F) == 4)
        return {{64, 1, 2}, {256, 4, 3}, {128, 2, 2}, {128, 1, 2}, {64, 2, 2}, {64, 1, 3}, {32, 1, 2}, {32, 1, 3}};
    return {{128, 1, 2}, {256, 2, 3}, {128, 2, 2}, {64, 1, 3}, {64, 1, 2}, {32, 1, 2}, {32, 1, 3}};
}

template <typename F>
class BatchImpl final : public BatchBase {
  public:
    BatchImpl(std::vector<SolverBase *> m, const ifl_batch_options &o) : m_(std::move(m)), opt_(o) {}
    ~BatchImpl() override { release(); }

    int init() {
        n_ = (int)m_.size();
        const ifl_params &p0 = m_[0]->params();
        variant_ = p0.variant;
        dev_ = p0.device;
        nq_ = variant_ >= IFL_HEAT ? 4 : 3;
        if (check(cudaSetDevice(dev_), "set device") ||
            check(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking), "stream"))
            return IFL_ERR_CUDA;
        for (cudaEvent_t *e : {&ev_step0_, &ev_step1_, &ev_pcg0_, &ev_pcg1_, &ev_heat0_, &ev_heat1_, &ev_trial0_,
                               &ev_trial1_})
            if (check(cudaEventCreate(e), "event")) return IFL_ERR_CUDA;
        member_ev_.resize(n_, nullptr);
        for (cudaEvent_t &e : member_ev_)
            if (check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event")) return IFL_ERR_CUDA;

        // device: scenes | bodies | tile_start | inflow_start | inflows | outs | flags | stats | sflags
        size_t off = 0;
        const size_t o_sc = off;
        off = al256(off + n_ * sizeof(Scene<F>));
        const size_t o_bd = off;
        off = al256(off + (size_t)n_ * kMaxBodies * sizeof(DevBody));
        const size_t o_ts = off;
        off = al256(off + (size_t)kTileShapes * (n_ + 1) * sizeof(int));
        const size_t o_is = off;
        off = al256(off + (n_ + 1) * sizeof(int));
        const size_t o_in = off;
        off = al256(off + (size_t)n_ * kMaxInflowRects * 4 * sizeof(BatchInflow));
        const size_t o_outs = off;
        off = al256(off + n_ * sizeof(PcgOut *));
        const size_t o_fl = off;
        off = al256(off + n_ * sizeof(unsigned *));
        const size_t o_st = off;
        off = al256(off + 2 * n_ * sizeof(PcgOut));
        const size_t o_sf = off;
        off = al256(off + n_ * sizeof(unsigned));
        dbytes_ = off;
        if (cudaMalloc(&d_, dbytes_) != cudaSuccess) {
            cudaGetLastError();
            d_ = nullptr;
            err_ = "device allocation of the batch tables failed";
            return IFL_ERR_NOMEM;
        }
        d_scenes_ = (Scene<F> *)(d_ + o_sc);
        d_bodies_ = (DevBody *)(d_ + o_bd);
        d_tile_start_ = (int *)(d_ + o_ts);
        d_inflow_start_ = (int *)(d_ + o_is);
        d_inflows_ = (BatchInflow *)(d_ + o_in);
        d_outs_ = (PcgOut **)(d_ + o_outs);
        d_flags_ = (unsigned **)(d_ + o_fl);
        d_stats_ = (PcgOut *)(d_ + o_st);
        d_sflags_ = (unsigned *)(d_ + o_sf);

        // pinned host staging: scenes | bodies | ctl | stats | sflags
        hbytes_ = al256(n_ * sizeof(Scene<F>)) + al256((size_t)n_ * kMaxBodies * sizeof(DevBody)) +
                  al256(n_ * sizeof(int4)) + al256(2 * n_ * sizeof(PcgOut)) + al256(n_ * sizeof(unsigned));
        if (cudaMallocHost(&h_, hbytes_) != cudaSuccess) {
            cudaGetLastError();
            h_ = nullptr;
            err_ = "pinned host allocation failed";
            return IFL_ERR_NOMEM;
        }
        h_scenes_ = (Scene<F> *)h_;
        h_bodies_ = (DevBody *)(h_ + al256(n_ * sizeof(Scene<F>)));
        h_ctl_ = (int4 *)((char *)h_bodies_ + al256((size_t)n_ * kMaxBodies * sizeof(DevBody)));
        h_stats_ = (PcgOut *)((char *)h_ctl_ + al256(n_ * sizeof(int4)));
        h_sflags_ = (unsigned *)((char *)h_stats_ + al256(2 * n_ * sizeof(PcgOut)));
        std::memset(h_stats_, 0, 2 * n_ * sizeof(PcgOut));
        std::memset(h_sflags_, 0, n_ * sizeof(unsigned));

        // static tables: the tile prefix sums of every candidate tile shape
        std::vector<int> ts((size_t)kTileShapes * (n_ + 1), 0);
        std::vector<PcgOut *> outs(n_);
        std::vector<unsigned *> fls(n_);
        for (int k = 0; k < kTileShapes; k++) {
            int *t = ts.data() + (size_t)k * (n_ + 1);
            for (int i = 0; i < n_; i++) t[i + 1] = t[i] + batch_tiles(scene(i).w, scene(i).h, kTileW[k], kTileH[k]);
        }
        for (int i = 0; i < n_; i++) {
            outs[i] = ((PcgScratch *)m_[i]->scratch_ptr())->out;
            fls[i] = scene(i).flags;
        }
        if (check(cudaMemcpy(d_tile_start_, ts.data(), ts.size() * sizeof(int), cudaMemcpyHostToDevice), "tables") ||
            check(cudaMemcpy(d_outs_, outs.data(), n_ * sizeof(PcgOut *), cudaMemcpyHostToDevice), "tables") ||
            check(cudaMemcpy(d_flags_, fls.data(), n_ * sizeof(unsigned *), cudaMemcpyHostToDevice), "tables"))
            return IFL_ERR_CUDA;
        inflows_.assign(n_, {});
        if (int e = upload_inflows()) return e;
        for (int k = 0; k < kTileShapes; k++) {
            SceneBatch<F> &b = tb_[k];
            b.scenes = d_scenes_;
            b.tile_start = d_tile_start_ + (size_t)k * (n_ + 1);
            b.inflows = d_inflows_;
            b.inflow_start = d_inflow_start_;
            b.n = n_;
            b.tiles = ts[(size_t)k * (n_ + 1) + n_];
            b.tw = kTileW[k];
            b.th = kTileH[k];
        }
        B_ = tb_[0];
        for (int p = 0; p < IFL_TILE_PHASES; p++) tile_pick_[p] = 0;
        if (opt_.tile_tune == 2) {
            for (int p = 0; p < IFL_TILE_ADVECT + 1; p++) tile_pick_[p] = tile_index(opt_.tile_w[p], opt_.tile_h[p]);
            tiles_tuned_ = true;
        } else if (opt_.tile_tune == 0) {
            tiles_tuned_ = true;
        }

        iters_.assign(n_, 0.0);
        for (int i = 0; i < n_; i++) {
            const Scene<F> &S = scene(i);
            iters_[i] = std::max(1.0, 0.6 * std::max(S.w, S.h));  // before the first solve
        }
        if (opt_.threads != 0) {
            PcgShape sh{opt_.threads, opt_.strips_per_block, opt_.stages};
            if (int e = make_plan(sh)) return e;
            tuned_ = true;
        }
        return IFL_OK;
    }

    int set_inflows(int member, const ifl_inflow *rects, int n) override {
        if (member < 0 || member >= n_ || n < 0 || n > kMaxInflowRects || (n > 0 && !rects)) return IFL_ERR_ARG;
        inflows_[member].assign(rects, rects + n);
        return upload_inflows();
    }

    int update(double dt) override {
        if (cudaSetDevice(dev_) != cudaSuccess) return fail_cuda("set device");
        // work the caller queued on a member's own stream comes first
        for (int i = 0; i < n_; i++)
            if (check(cudaEventRecord(member_ev_[i], m_[i]->stream()), "member event") ||
                check(cudaStreamWaitEvent(st_, member_ev_[i], 0), "member wait"))
                return IFL_ERR_CUDA;
        if (int e = stage_tables()) return e;
        if (!tiles_tuned_) {
            if (int e = autotune_tiles(dt)) return e;
            tiles_tuned_ = true;
        }
        if (!tuned_) {
            if (int e = autotune(dt)) return e;
            tuned_ = true;
        }
        if (int e = schedule()) return e;
        if (int e = upload_ctl()) return e;
        int e = IFL_OK;
        if (opt_.use_graph && graph_ok_) {
            if (!gexec_ || graph_dt_ != dt) e = capture(dt);
            if (e == IFL_OK && gexec_) {
                if (check(cudaGraphLaunch(gexec_, st_), "graph launch")) return IFL_ERR_CUDA;
                launches_ += launches_per_step_;
            }
        }
        if (!(opt_.use_graph && graph_ok_ && gexec_)) {
            e = record_step(dt, true);
            if (e) return e;
        }
        if (check(cudaStreamSynchronize(st_), "batch step")) return IFL_ERR_CUDA;
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, ev_step0_, ev_step1_) == cudaSuccess) last_step_ms_ = ms;
        double pcg = 0.0;
        if (cudaEventElapsedTime(&ms, ev_pcg0_, ev_pcg1_) == cudaSuccess) pcg += ms;
        if (variant_ >= IFL_HEAT && cudaEventElapsedTime(&ms, ev_heat0_, ev_heat1_) == cudaSuccess) pcg += ms;
        last_pcg_ms_ = pcg;
        cudaGetLastError();
        bool timeout = false;
        for (int i = 0; i < n_; i++) {
            iters_[i] = std::max(1, h_stats_[2 * i].iterations + h_stats_[2 * i + 1].iterations);
            if (h_sflags_[i] & FLAG_TIMEOUT) timeout = true;
            for (int q = 0; q < 4; q++)
                if (m_[i]->has_quantity(q)) m_[i]->flip(q);
            m_[i]->count_step();
        }
        steps_++;
        if (timeout) {
            err_ = "a bounded device-side wait timed out";
            return IFL_ERR_TIMEOUT;
        }
        return IFL_OK;
    }

    int get_stats(ifl_step_stats *out, int n) override {
        if (!out || n != n_) return IFL_ERR_ARG;
        for (int i = 0; i < n_; i++) {
            const PcgOut &a = h_stats_[2 * i], &b = h_stats_[2 * i + 1];
            out[i].pressure = {a.iterations, a.status, a.max_error};
            out[i].heat = {b.iterations, b.status, b.max_error};
            out[i].device_flags = h_sflags_[i];
            out[i].steps = (uint32_t)steps_;
        }
        return IFL_OK;
    }

    int info(ifl_batch_info *o) override {
        std::memset(o, 0, sizeof *o);
        o->members = n_;
        o->threads = shape_.threads;
        o->strips_per_block = shape_.K;
        o->stages = shape_.stages;
        o->grid = plan_ ? pcg_batch_grid(plan_) : 0;
        o->graph = (opt_.use_graph && graph_ok_ && gexec_) ? 1 : 0;
        o->candidates = (int)trial_ms_.size();
        for (size_t i = 0; i < trial_ms_.size() && i < 8; i++) o->candidate_ms[i] = trial_ms_[i];
        o->last_step_ms = last_step_ms_;
        o->last_pcg_ms = last_pcg_ms_;
        o->launches = launches_;
        o->steps = steps_;
        o->h2d_bytes_last_step = h2d_bytes_;
        o->d2h_bytes_last_step = (int64_t)(2 * n_ * sizeof(PcgOut) + n_ * sizeof(unsigned));
        for (int p = 0; p < IFL_TILE_PHASES; p++) {
            o->tile_w[p] = kTileW[tile_pick_[p]];
            o->tile_h[p] = kTileH[tile_pick_[p]];
            o->tile_ms[p] = tile_ms_[p];
        }
        return IFL_OK;
    }

    cudaStream_t stream() const override { return st_; }
    int device() const override { return dev_; }

  private:
    const Scene<F> &scene(int i) const { return *(const Scene<F> *)m_[i]->scene_ptr(); }

    bool check(cudaError_t e, const char *what) {
        if (e == cudaSuccess) return false;
        err_ = std::string(what) + ": " + cudaGetErrorString(e);
        return true;
    }
    int fail_cuda(const char *what) {
        check(cudaGetLastError(), what);
        return IFL_ERR_CUDA;
    }

    int upload_inflows() {
        std::vector<int> start(n_ + 1, 0);
        std::vector<BatchInflow> recs;
        for (int i = 0; i < n_; i++) {
            for (const ifl_inflow &r : inflows_[i]) {
                const double val[4] = {r.d, r.t, r.u, r.v};
                for (int q = 0; q < 4; q++) {
                    if (!m_[i]->has_quantity(q)) continue;
                    BatchInflow b;
                    b.q = q;
                    b.pad_ = 0;
                    b.x0 = r.x;
                    b.y0 = r.y;
                    b.x1 = r.x + r.w;
                    b.y1 = r.y + r.h;
                    b.val = val[q];
                    recs.push_back(b);
                }
            }
            start[i + 1] = (int)recs.size();
        }
        if (check(cudaStreamSynchronize(st_), "inflow sync") ||
            check(cudaMemcpy(d_inflow_start_, start.data(), start.size() * sizeof(int), cudaMemcpyHostToDevice),
                  "inflows") ||
            (!recs.empty() && check(cudaMemcpy(d_inflows_, recs.data(), recs.size() * sizeof(BatchInflow),
                                               cudaMemcpyHostToDevice),
                                    "inflows")))
            return IFL_ERR_CUDA;
        return IFL_OK;
    }

    // Scene table (current source/destination pointers, bodies) and bodies.
    int stage_tables() {
        size_t nb = 0;
        for (int i = 0; i < n_; i++) {
            Scene<F> S = scene(i);
            const std::vector<ifl_body> &bodies = m_[i]->bodies();
            S.bodies = d_bodies_ + nb;
            S.nbodies = variant_ >= IFL_SOLID ? (int)bodies.size() : 0;
            for (size_t k = 0; k < bodies.size(); k++) to_dev_body(bodies[k], h_bodies_[nb + k]);
            nb += bodies.size();
            h_scenes_[i] = S;
            const ifl_params &p = m_[i]->params();
            h_ctl_[i] = make_int4(m_[i]->pinned_pressure(), m_[i]->pinned_heat(), p.max_iter_pressure,
                                  p.max_iter_heat);
        }
        h2d_bytes_ = (int64_t)(n_ * sizeof(Scene<F>) + nb * sizeof(DevBody) + n_ * sizeof(int4)) +
                     (plan_ ? pcg_batch_table_bytes(plan_) : 0);
        if (check(cudaMemcpyAsync(d_scenes_, h_scenes_, n_ * sizeof(Scene<F>), cudaMemcpyHostToDevice, st_),
                  "scene table") ||
            (nb && check(cudaMemcpyAsync(d_bodies_, h_bodies_, nb * sizeof(DevBody), cudaMemcpyHostToDevice, st_),
                         "body table")))
            return IFL_ERR_CUDA;
        return IFL_OK;
    }

    int upload_ctl() {
        return check(cudaMemcpyAsync(pcg_batch_ctl(plan_), h_ctl_, n_ * sizeof(int4), cudaMemcpyHostToDevice, st_),
                     "pcg control")
                   ? IFL_ERR_CUDA
                   : IFL_OK;
    }

    // Estimated PCG time of each scene: iterations x (two wavefront sweeps,
    // D + lag per strip steps each; the elementwise passes over its team).
    // Estimated time (microseconds) of scene i's solve on a team of g blocks:
    // per PCG iteration a forward and a backward sweep, the elementwise passes
    // and the team barriers.  A sweep of S strips by P = g*K warps (strips taken
    // round-robin) finishes after
    //   max((S-1)*lag + D*tau, (S-1)/P * D*tau + ((S-1) mod P)*lag + D*tau):
    // strip s starts a hand-over (lag) after strip s-1 and not before its warp
    // finished strip s-P.  The elementwise passes cost a fixed time per cell
    // and warp; a team of more than one block adds its barriers, which grow
    // with its size.  Constants fitted to per-phase timers in the batched
    // kernel on GB300 (512-scene batch, FP32 form, 64-thread blocks, teams of
    // 1 to 64 blocks): tau = 0.11 us per wavefront step, lag = 6.4 us per
    // strip, 27.4 ns per cell per two-warp block for three elementwise passes,
    // barriers 15 + 6 log2(g) us for five team barriers per iteration; the
    // sigma pass (about an eighth of the elementwise time) and one barrier have
    // since moved into the forward sweep, leaving 24 ns and 12 + 4.8 log2(g).
    // The step time is flat around these values: with the faster matvec that
    // followed, 17, 20 or 30 ns per cell and a lag of 8 us changed the
    // 512-scene step by less than its step-to-step spread.
    double plan_cost(int i, int g) const {
        constexpr double kTau = 0.11, kLag = 6.4, kElemNs = 24.0;
        const Scene<F> &S = scene(i);
        const int P = g * shape_.K, Sn = S.sd.S;
        const double Dt = S.sd.D * kTau * (sizeof(F) == 8 ? 3.0 : 1.0);
        const double sweep = std::max((Sn - 1) * kLag + Dt, ((Sn - 1) / P) * Dt + ((Sn - 1) % P) * kLag + Dt);
        const double elem = 1e-3 * kElemNs * (double)S.w * S.h / g * (64.0 / shape_.threads);
        const double bars = g == 1 ? 1.6 : 12.0 + 4.8 * std::log2((double)g);
        return iters_[i] * (2.0 * sweep + elem + bars);
    }

    int schedule() {
        // Each scene starts in the class of the smallest team that gives each
        // of its strips its own sweeping warp; the planner then adds teams or
        // doubles team sizes where the finish time needs them.  (Choosing
        // smaller, round-robin teams for the step time the grid could hold
        // spent fewer block-microseconds but packed worse on GB300: 1.12-1.24 s
        // against 1.00 s per step of the 512-scene batch.)
        std::vector<int> cls(n_);
        for (int i = 0; i < n_; i++) {
            const int cover = pow2ceil((scene(i).sd.S + shape_.K - 1) / shape_.K);
            int c = 0;
            while ((1 << c) < cover && (1 << c) < 128) c++;
            cls[i] = c;
        }
        const PlanWork work = [this](int i, int g) { return plan_cost(i, g); };
        if (pcg_batch_schedule(plan_, cls.data(), work, st_) != 0) {
            err_ = "batched PCG schedule failed";
            return IFL_ERR_CUDA;
        }
        return IFL_OK;
    }

    int make_plan(const PcgShape &sh) {
        std::vector<const Scene<F> *> sc(n_);
        std::vector<const PcgScratch *> sx(n_);
        for (int i = 0; i < n_; i++) {
            sc[i] = &scene(i);
            sx[i] = (const PcgScratch *)m_[i]->scratch_ptr();
        }
        std::string why;
        PcgBatchPlan *P = pcg_batch_create<F>(sc.data(), sx.data(), n_, sh, &why);
        if (P) pcg_batch_set_max_team(P, opt_.max_team_blocks);
        if (!P) {
            err_ = "batched PCG shape {" + std::to_string(sh.threads) + "," + std::to_string(sh.K) + "," +
                   std::to_string(sh.stages) + "}: " + why;
            return IFL_ERR_UNSUPPORTED;
        }
        if (plan_) {
            cudaStreamSynchronize(st_);
            pcg_batch_destroy(plan_);
        }
        plan_ = P;
        shape_ = sh;
        destroy_graph();
        return IFL_OK;
    }

    int pcg(int heat) {
        PcgConfig cfg{PCG_FACTOR | PCG_SOLVE, 0, -2, heat};
        cfg.wait_limit = m_[0]->wait_limit();  // the launch waits with its first member's limit
        if (check(launch_pcg_batch<F>(plan_, cfg, st_), "batched PCG launch")) return IFL_ERR_CUDA;
        launches_++;
        return IFL_OK;
    }

    // The phases before the first PCG solve of a step.
    void record_head(double dt) {
        launch_batch_inflow<F>(B_, st_);
        launches_++;
        if (variant_ >= IFL_SOLID) {
            launch_batch_fill_solid<F>(TB(IFL_TILE_FILL), variant_, nq_, st_);
            launches_ += variant_ >= IFL_CURVED ? 2 : 1;
        }
        if (variant_ >= IFL_HEAT) {
            launch_batch_heat_assemble<F>(TB(IFL_TILE_HEAT_ASSEMBLE), dt, st_);
            launches_++;
        } else {
            if (variant_ >= IFL_SOLID) {
                launch_batch_bc<F>(TB(IFL_TILE_BC), st_);
                launches_++;
            }
            launch_batch_assemble<F>(TB(IFL_TILE_ASSEMBLE), dt, ASM_RHS | ASM_MATRIX, st_);
            launches_++;
        }
    }

    int record_step(double dt, bool timed) {
        const int64_t l0 = launches_;
        // inside a capture the records must become event nodes of the graph
        const unsigned ext = capturing_ ? cudaEventRecordExternal : cudaEventRecordDefault;
        if (timed && check(cudaEventRecordWithFlags(ev_step0_, st_, ext), "event")) return IFL_ERR_CUDA;
        record_head(dt);
        if (variant_ >= IFL_HEAT) {
            if (timed) cudaEventRecordWithFlags(ev_heat0_, st_, ext);
            if (int e = pcg(1)) return e;
            if (timed) cudaEventRecordWithFlags(ev_heat1_, st_, ext);
            launch_batch_heat_to_rows<F>(B_, st_);
            launch_batch_extrapolate<F>(B_, 1u << 1, st_);
            launch_batch_buoyancy<F>(B_, dt, st_);
            launch_batch_bc<F>(TB(IFL_TILE_BC), st_);
            launch_batch_assemble<F>(TB(IFL_TILE_ASSEMBLE), dt,
                                     ASM_RHS | ASM_MATRIX | (variant_ >= IFL_VARDENS ? ASM_DENS : 0), st_);
            launches_ += 1 + 3 + 1 + 1 + 1;
        }
        if (timed) cudaEventRecordWithFlags(ev_pcg0_, st_, ext);
        if (int e = pcg(0)) return e;
        if (timed) cudaEventRecordWithFlags(ev_pcg1_, st_, ext);
        launch_batch_apply_pressure<F>(B_, dt, st_);
        launches_++;
        if (variant_ >= IFL_SOLID) {
            launch_batch_extrapolate<F>(B_, (1u << 0) | (1u << 2) | (1u << 3), st_);
            launch_batch_bc<F>(TB(IFL_TILE_BC), st_);
            launches_ += 4;
        }
        launch_batch_advect<F>(TB(IFL_TILE_ADVECT), dt, st_);
        gather_stats_kernel<<<(n_ + 127) / 128, 128, 0, st_>>>(d_outs_, d_flags_, d_stats_, d_sflags_, n_);
        launches_ += 2;
        if (check(cudaMemcpyAsync(h_stats_, d_stats_, 2 * n_ * sizeof(PcgOut), cudaMemcpyDeviceToHost, st_),
                  "stats") ||
            check(cudaMemcpyAsync(h_sflags_, d_sflags_, n_ * sizeof(unsigned), cudaMemcpyDeviceToHost, st_),
                  "stats"))
            return IFL_ERR_CUDA;
        if (timed && check(cudaEventRecordWithFlags(ev_step1_, st_, ext), "event")) return IFL_ERR_CUDA;
        launches_per_step_ = launches_ - l0;
        return check(cudaGetLastError(), "batch step") ? IFL_ERR_CUDA : IFL_OK;
    }

    void destroy_graph() {
        if (gexec_) cudaGraphExecDestroy(gexec_);
        gexec_ = nullptr;
    }

    int capture(double dt) {
        destroy_graph();
        cudaGraph_t g = nullptr;
        const int64_t l0 = launches_;
        if (check(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal), "begin capture")) {
            graph_ok_ = false;
            cudaGetLastError();
            return IFL_OK;
        }
        capturing_ = true;
        int e = record_step(dt, true);
        capturing_ = false;
        cudaError_t ce = cudaStreamEndCapture(st_, &g);
        launches_ = l0;  // counted again at every replay
        if (e != IFL_OK || ce != cudaSuccess || !g || cudaGraphInstantiate(&gexec_, g, 0) != cudaSuccess) {
            // capture unsupported for this sequence: run the launches directly
            cudaGetLastError();
            if (g) cudaGraphDestroy(g);
            gexec_ = nullptr;
            graph_ok_ = false;
            return IFL_OK;
        }
        cudaGraphDestroy(g);
        graph_dt_ = dt;
        return IFL_OK;
    }

    const SceneBatch<F> &TB(int phase) const { return tb_[tile_pick_[phase]]; }

    static int tile_index(int w, int h) {
        for (int k = 0; k < kTileShapes; k++)
            if (kTileW[k] == w && kTileH[k] == h) return k;
        return -1;
    }

    // One launch of a tuned phase with tile shape k (the phase's arguments of
    // this variant's step); false if the variant has no such phase.
    bool tile_trial(int phase, int k, double dt) {
        const SceneBatch<F> &b = tb_[k];
        switch (phase) {
        case IFL_TILE_FILL:
            if (variant_ < IFL_SOLID) return false;
            launch_batch_fill_solid<F>(b, variant_, nq_, st_);
            launches_ += variant_ >= IFL_CURVED ? 2 : 1;
            return true;
        case IFL_TILE_BC:
            if (variant_ < IFL_SOLID) return false;
            launch_batch_bc<F>(b, st_);
            break;
        case IFL_TILE_ASSEMBLE:
            launch_batch_assemble<F>(b, dt, ASM_RHS | ASM_MATRIX | (variant_ >= IFL_VARDENS ? ASM_DENS : 0), st_);
            break;
        case IFL_TILE_HEAT_ASSEMBLE:
            if (variant_ < IFL_HEAT) return false;
            launch_batch_heat_assemble<F>(b, dt, st_);
            break;
        case IFL_TILE_ADVECT:
            launch_batch_advect<F>(b, dt, st_);
            break;
        default:
            return false;
        }
        launches_++;
        return true;
    }

    // Tile shapes of the tuned phases: each candidate runs each phase twice on
    // the current state (the faster run counts).  These phases are idempotent:
    // they write only what the step rewrites before reading it (solid fields,
    // boundary velocities, the systems and right-hand sides, the advected
    // copies), and the step that follows runs every one of them again.
    int autotune_tiles(double dt) {
        for (int p = 0; p <= IFL_TILE_ADVECT; p++) {
            double best = std::numeric_limits<double>::infinity();
            for (int k = 0; k < kTileShapes; k++) {
                double t = std::numeric_limits<double>::infinity();
                for (int rep = 0; rep < 2; rep++) {
                    if (check(cudaEventRecord(ev_trial0_, st_), "event")) return IFL_ERR_CUDA;
                    if (!tile_trial(p, k, dt)) break;
                    if (check(cudaEventRecord(ev_trial1_, st_), "event") ||
                        check(cudaEventSynchronize(ev_trial1_), "tile autotune"))
                        return IFL_ERR_CUDA;
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, ev_trial0_, ev_trial1_);
                    t = std::min(t, (double)ms);
                }
                if (t < best) {
                    best = t;
                    tile_pick_[p] = k;
                }
            }
            tile_ms_[p] = best < std::numeric_limits<double>::infinity() ? best : 0.0;
        }
        return check(cudaGetLastError(), "tile autotune") ? IFL_ERR_CUDA : IFL_OK;
    }

    // Each candidate shape solves the first step's real system with a pinned
    // iteration count (twice; the faster run counts).  The phases before the
    // first solve are idempotent, so the real step repeats them unchanged.
    int autotune(double dt) {
        const int iters = opt_.tune_iterations > 0 ? opt_.tune_iterations : 8;
        const int heat = variant_ >= IFL_HEAT ? 1 : 0;
        record_head(dt);
        double best = std::numeric_limits<double>::infinity();
        PcgShape best_sh{};
        trial_ms_.clear();
        for (const PcgShape &sh : candidate_shapes<F>()) {
            if (make_plan(sh) != IFL_OK) {
                trial_ms_.push_back(-1.0);
                continue;
            }
            if (int e = schedule()) return e;
            if (int e = upload_ctl()) return e;
            double t = std::numeric_limits<double>::infinity();
            for (int rep = 0; rep < 2; rep++) {
                PcgConfig cfg{PCG_FACTOR | PCG_SOLVE, 0, iters, heat};
                if (check(cudaEventRecord(ev_trial0_, st_), "event") ||
                    check(launch_pcg_batch<F>(plan_, cfg, st_), "autotune launch") ||
                    check(cudaEventRecord(ev_trial1_, st_), "event") ||
                    check(cudaEventSynchronize(ev_trial1_), "autotune"))
                    return IFL_ERR_CUDA;
                launches_++;
                float ms = 0.f;
                cudaEventElapsedTime(&ms, ev_trial0_, ev_trial1_);
                t = std::min(t, (double)ms);
            }
            trial_ms_.push_back(t);
            if (t < best) {
                best = t;
                best_sh = sh;
            }
        }
        if (!(best < std::numeric_limits<double>::infinity())) {
            err_ = "no batched PCG shape fits this batch";
            return IFL_ERR_UNSUPPORTED;
        }
        const double home = trial_ms_.empty() ? -1.0 : trial_ms_[0];
        if (home > 0.0 && home <= best * (1.0 + kHomeMargin)) best_sh = candidate_shapes<F>()[0];
        return make_plan(best_sh);
    }

    void release() {
        if (st_) cudaStreamSynchronize(st_);
        destroy_graph();
        if (plan_) pcg_batch_destroy(plan_);
        plan_ = nullptr;
        for (cudaEvent_t e : member_ev_)
            if (e) cudaEventDestroy(e);
        member_ev_.clear();
        for (cudaEvent_t e : {ev_step0_, ev_step1_, ev_pcg0_, ev_pcg1_, ev_heat0_, ev_heat1_, ev_trial0_,
                              ev_trial1_})
            if (e) cudaEventDestroy(e);
        if (h_) cudaFreeHost(h_);
        h_ = nullptr;
        if (d_) cudaFree(d_);
        d_ = nullptr;
        if (st_) cudaStreamDestroy(st_);
        st_ = nullptr;
    }

    std::vector<SolverBase *> m_;
    ifl_batch_options opt_;
    int n_ = 0, variant_ = 0, nq_ = 3, dev_ = 0;
    cudaStream_t st_ = nullptr;
    std::vector<cudaEvent_t> member_ev_;
    cudaEvent_t ev_step0_ = nullptr, ev_step1_ = nullptr, ev_pcg0_ = nullptr, ev_pcg1_ = nullptr;
    cudaEvent_t ev_heat0_ = nullptr, ev_heat1_ = nullptr, ev_trial0_ = nullptr, ev_trial1_ = nullptr;
    char *d_ = nullptr;
    size_t dbytes_ = 0;
    Scene<F> *d_scenes_ = nullptr;
    DevBody *d_bodies_ = nullptr;
    int *d_tile_start_ = nullptr, *d_inflow_start_ = nullptr;
    BatchInflow *d_inflows_ = nullptr;
    PcgOut **d_outs_ = nullptr;
    unsigned **d_flags_ = nullptr;
    PcgOut *d_stats_ = nullptr;
    unsigned *d_sflags_ = nullptr;
    char *h_ = nullptr;
    size_t hbytes_ = 0;
    Scene<F> *h_scenes_ = nullptr;
    DevBody *h_bodies_ = nullptr;
    int4 *h_ctl_ = nullptr;
    PcgOut *h_stats_ = nullptr;
    unsigned *h_sflags_ = nullptr;
    std::vector<std::vector<ifl_inflow>> inflows_;
    SceneBatch<F> B_{};                 // 32 x 8 tiles (the phases that are not tuned)
    SceneBatch<F> tb_[kTileShapes]{};   // the same tables for every candidate tile shape
    int tile_pick_[IFL_TILE_PHASES]{};  // candidate in use per IFL_TILE_* phase
    double tile_ms_[IFL_TILE_PHASES]{};
    bool tiles_tuned_ = false;
    PcgBatchPlan *plan_ = nullptr;
    PcgShape shape_{};
    bool tuned_ = false;
    std::vector<double> iters_, trial_ms_;
    cudaGraphExec_t gexec_ = nullptr;
    double graph_dt_ = std::numeric_limits<double>::quiet_NaN();
    bool graph_ok_ = true, capturing_ = false;
    int64_t launches_ = 0, launches_per_step_ = 0, steps_ = 0;
    double last_step_ms_ = 0.0, last_pcg_ms_ = 0.0;
    int64_t h2d_bytes_ = 0;
};

}  // namespace

int make_batch(SolverBase *const *members, int n, const ifl_batch_options &opt, std::unique_ptr<BatchBase> *out,
               std::string *err) {
    if (!members || n <= 0 || !out) return IFL_ERR_ARG;
    const ifl_params &p0 = members[0]->params();
    for (int i = 0; i < n; i++) {
        if (!members[i]) return IFL_ERR_ARG;
        const ifl_params &p = members[i]->params();
        if (p.variant == IFL_FLIP || p.variant <= IFL_GS) {
            if (err) *err = "step 1, 2 and 8 handles are stepped one by one, not in batches";
            return IFL_ERR_UNSUPPORTED;
        }
        if (p.variant != p0.variant || p.precision != p0.precision || p.device != p0.device) {
            if (err) *err = "batch members differ in variant, precision or device";
            return IFL_ERR_ARG;
        }
        for (int j = 0; j < i; j++)
            if (members[j] == members[i]) {
                if (err) *err = "a handle appears twice in the batch";
                return IFL_ERR_ARG;
            }
    }
    if (opt.threads != 0 && opt.threads != 32 && opt.threads != 64 && opt.threads != 128 && opt.threads != 256)
        return IFL_ERR_ARG;
    if (opt.max_team_blocks < 0) return IFL_ERR_ARG;
    if (opt.tile_tune < 0 || opt.tile_tune > 2) return IFL_ERR_ARG;
    if (opt.tile_tune == 2)
        for (int p = 0; p <= IFL_TILE_ADVECT; p++) {
            bool ok = false;
            for (int k = 0; k < kTileShapes; k++) ok = ok || (opt.tile_w[p] == kTileW[k] && opt.tile_h[p] == kTileH[k]);
            if (!ok) {
                if (err) *err = "tile shape " + std::to_string(opt.tile_w[p]) + "x" + std::to_string(opt.tile_h[p]) +
                                " is not a candidate";
                return IFL_ERR_ARG;
            }
        }
    std::vector<SolverBase *> m(members, members + n);
    int e;
    if (p0.precision == IFL_FP32) {
        auto *b = new BatchImpl<float>(std::move(m), opt);
        out->reset(b);
        e = b->init();
    } else {
        auto *b = new BatchImpl<double>(std::move(m), opt);
        out->reset(b);
        e = b->init();
    }
    if (e != IFL_OK) {
        if (err) *err = (*out)->error();
        out->reset();
    }
    return e;
}

}  // namespace ifl
