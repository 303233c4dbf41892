// solver.cu - host-side FluidSolver: device arena, phase orchestration and
// field transfer behind the C ABI (include/ifluids.h).  No kernels live here.
//
// update() follows FluidSolver::update of the reference step selected by the
// variant (1-matrixless/Fluid.cpp:284-297, 3-conjugate-gradients/Fluid.cpp:433-447, 4-solid-boundaries/Fluid.cpp:869-895,
// 5-curved-boundaries/Fluid.cpp:927-953, 6-heat/Fluid.cpp:966-1006,
// 7-variable-density/Fluid.cpp:995-1034, 8-flip/Fluid.cpp:1350-1413); buildRhs/computeDensities/
// buildPressureMatrix run as one assembly launch and buildPreconditioner +
// project as one persistent PCG launch.
#include "solver.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <type_traits>
#include <cstdio>
#include <cstring>
#include <vector>

namespace ifl {

namespace {

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

struct Carver {
    size_t off = 0;
    template <typename T>
    T *take(char *base, size_t count) {
        off = align_up(off, 256);
        T *p = base ? (T *)(base + off) : nullptr;
        off += count * sizeof(T);
        return p;
    }
};

}  // namespace

template <typename F>
class SolverImpl final : public SolverBase {
  public:
    explicit SolverImpl(const ifl_params &prm) : SolverBase(prm) {}
    ~SolverImpl() override { release(); }

    // Device bytes init() allocates for these parameters (no GPU work).
    static size_t arena_size(const ifl_params &prm, int max_blocks) {
        SolverImpl s(prm);
        s.P_ = (int)align_up((size_t)prm.w + 2, 32);
        s.rows_ = prm.h + 2;
        s.nq_ = prm.variant >= IFL_HEAT ? 4 : 3;
        s.max_blocks_ = max_blocks;
        Carver c;
        s.carve(nullptr, c);
        return c.off;
    }

    int init() override {
        const int w = prm_.w, h = prm_.h;
        if (check(cudaSetDevice(prm_.device), "set device")) return IFL_ERR_CUDA;
        P_ = (int)align_up((size_t)w + 2, 32);
        rows_ = h + 2;
        nq_ = prm_.variant >= IFL_HEAT ? 4 : 3;
        if (prm_.stream) {
            stream_ = (cudaStream_t)prm_.stream;
        } else {
            if (check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "stream")) return IFL_ERR_CUDA;
            own_stream_ = true;
        }
        max_blocks_ = pcg_max_blocks<F>();
        Carver c;
        carve(nullptr, c);
        arena_bytes_ = c.off;
        cudaError_t e = cudaMalloc(&arena_, arena_bytes_);
        if (e != cudaSuccess) {
            arena_ = nullptr;
            cudaGetLastError();
            err_ = "device allocation of " + std::to_string(arena_bytes_) + " bytes failed";
            return IFL_ERR_NOMEM;
        }
        Carver c2;
        carve((char *)arena_, c2);
        if (check(cudaMemsetAsync(arena_, 0, arena_bytes_, stream_), "memset")) return IFL_ERR_CUDA;
        // FluidQuantity ctor: volume = 1 (5-curved-boundaries and later),
        // temperature = ambient (6-heat/Fluid.cpp:935-938).
        if (prm_.variant >= IFL_CURVED) {
            std::vector<double> ones((size_t)P_ * rows_, 1.0);
            for (int q = 0; q < 4; q++)
                if (present(q) && S_.q[q].vol)
                    if (check(cudaMemcpy(S_.q[q].vol, ones.data(), ones.size() * 8, cudaMemcpyHostToDevice),
                              "init volume"))
                        return IFL_ERR_CUDA;
        }
        if (prm_.variant >= IFL_HEAT) {
            std::vector<F> tamb((size_t)P_ * rows_, (F)294.0);
            if (check(cudaMemcpy(S_.q[1].src, tamb.data(), tamb.size() * sizeof(F), cudaMemcpyHostToDevice),
                      "init T"))
                return IFL_ERR_CUDA;
        }
        if (prm_.variant == IFL_FLIP) {
            int ctl[FC_WORDS] = {};
            ctl[FC_RNG] = (int)0xBA5EBA11u;  // frand's seed, 8-flip/Fluid.cpp:39
            if (check(cudaMemcpy(X_.ctl, ctl, sizeof ctl, cudaMemcpyHostToDevice), "flip state")) return IFL_ERR_CUDA;
        }
        if (check(cudaStreamSynchronize(stream_), "init sync")) return IFL_ERR_CUDA;
        return IFL_OK;
    }

    // ----------------------------------------------------------- phases
    int add_inflow(double x, double y, double w, double h, double d, double t, double u, double v) override {
        if (prm_.variant == IFL_FLIP) {  // applied inside the next update, after copy()
            pending_.push_back({x, y, w, h, d, t, u, v});
            return IFL_OK;
        }
        const double val[4] = {d, t, u, v};
        for (int q = 0; q < 4; q++) {
            if (!present(q)) continue;
            int t = tbegin(IFL_K_FACES);
            launch_inflow<F>(S_, q, x, y, x + w, y + h, val[q], stream_);
            tend(t);
            launches_++;
        }
        return launch_check("inflow");
    }

    int run_phase(int ph, double dt) override {
        const int var = prm_.variant;
        switch (ph) {
        case IFL_PH_FILL_SOLID:
            if (var >= IFL_SOLID && !bodies_.empty()) {
                if (int e = upload_bodies()) return e;
                int t = tbegin(IFL_K_SOLID);
                launch_fill_solid<F>(S_, stream_);
                tend(t);
                launches_ += var >= IFL_CURVED ? 2 : 1;
            }
            break;
        case IFL_PH_HEAT:
            if (var >= IFL_HEAT) return heat_solve(dt);
            break;
        case IFL_PH_EXTRAP_T:
            if (var >= IFL_HEAT) extrapolate(1u << 1);
            break;
        case IFL_PH_BUOYANCY:
            if (var >= IFL_HEAT) {
                int t = tbegin(IFL_K_FACES);
                launch_buoyancy<F>(S_, dt, stream_);
                tend(t);
                launches_++;
            }
            break;
        case IFL_PH_BC:
            if (var >= IFL_SOLID) {
                int t = tbegin(IFL_K_FACES);
                launch_bc<F>(S_, stream_);
                tend(t);
                launches_++;
            }
            break;
        case IFL_PH_RHS: assemble(dt, ASM_RHS); break;
        case IFL_PH_DENSITIES:
            if (var >= IFL_VARDENS) assemble(dt, ASM_DENS);
            break;
        case IFL_PH_MATRIX:
            if (var > IFL_GS) assemble(dt, ASM_MATRIX);
            break;
        case IFL_PH_PRECON:
            if (var > IFL_GS) return pcg(PCG_FACTOR, false);
            break;
        case IFL_PH_PROJECT:
            if (var <= IFL_GS) return gauss_seidel(dt);
            return pcg(PCG_SOLVE, false);
        case IFL_PH_APPLY_P: {
            int t = tbegin(IFL_K_FACES);
            launch_apply_pressure<F>(S_, dt, stream_);
            tend(t);
            launches_++;
            break;
        }
        case IFL_PH_EXTRAP_DUV:
            if (var >= IFL_SOLID) extrapolate((1u << 0) | (1u << 2) | (1u << 3));
            break;
        case IFL_PH_P2G:
        case IFL_PH_FLIP_COPY:
        case IFL_PH_G2P:
        case IFL_PH_PADVECT:
            if (var == IFL_FLIP) return flip_phase(ph, dt);
            break;
        case IFL_PH_ADVECT: {
            if (var == IFL_FLIP) break;  // particles carry the quantities instead
            int t = tbegin(IFL_K_ADVECT);
            launch_advect<F>(S_, dt, stream_);
            tend(t);
            launches_++;
            for (int q = 0; q < 4; q++)
                if (present(q)) std::swap(S_.q[q].src, S_.q[q].dst);
            break;
        }
        default: return IFL_ERR_ARG;
        }
        return launch_check("phase");
    }

    int update(double dt) override {
        const int var = prm_.variant;
        int e;
        if (var == IFL_FLIP) {  // 8-flip/Fluid.cpp:1350-1413
            static const int order[] = {IFL_PH_FILL_SOLID, IFL_PH_P2G, IFL_PH_FLIP_COPY, IFL_PH_HEAT,
                                        IFL_PH_EXTRAP_T, IFL_PH_BUOYANCY, IFL_PH_BC};
            for (int ph : order)
                if ((e = run_phase(ph, dt))) return e;
            assemble(dt, ASM_RHS | ASM_MATRIX | ASM_DENS);
            if ((e = pcg(PCG_FACTOR | PCG_SOLVE, false))) return e;
            static const int tail[] = {IFL_PH_APPLY_P, IFL_PH_EXTRAP_DUV, IFL_PH_BC, IFL_PH_G2P, IFL_PH_PADVECT};
            for (int ph : tail)
                if ((e = run_phase(ph, dt))) return e;
        } else if (var <= IFL_GS) {  // 1-matrixless/Fluid.cpp:284-297
            assemble(dt, ASM_RHS);
            if ((e = gauss_seidel(dt))) return e;
            if ((e = run_phase(IFL_PH_APPLY_P, dt))) return e;
            if ((e = run_phase(IFL_PH_ADVECT, dt))) return e;
        } else if (var == IFL_PLAIN) {
            assemble(dt, ASM_RHS | ASM_MATRIX);
            if ((e = pcg(PCG_FACTOR | PCG_SOLVE, false))) return e;
            if ((e = run_phase(IFL_PH_APPLY_P, dt))) return e;
            if ((e = run_phase(IFL_PH_ADVECT, dt))) return e;
        } else {
            if ((e = run_phase(IFL_PH_FILL_SOLID, dt))) return e;
            if (var >= IFL_HEAT) {
                if ((e = heat_solve(dt))) return e;
                extrapolate(1u << 1);
                if ((e = run_phase(IFL_PH_BUOYANCY, dt))) return e;
            }
            if ((e = run_phase(IFL_PH_BC, dt))) return e;
            assemble(dt, ASM_RHS | ASM_MATRIX | (var >= IFL_VARDENS ? ASM_DENS : 0));
            if ((e = pcg(PCG_FACTOR | PCG_SOLVE, false))) return e;
            if ((e = run_phase(IFL_PH_APPLY_P, dt))) return e;
            extrapolate((1u << 0) | (1u << 2) | (1u << 3));
            if ((e = run_phase(IFL_PH_BC, dt))) return e;
            if ((e = run_phase(IFL_PH_ADVECT, dt))) return e;
        }
        steps_++;
        return launch_check("update");
    }

    // ------------------------------------------------------ field access
    SDIdx sd_index() const override { return S_.sd; }

    int field_info(int field, void **ptr, int *elem, int *w, int *h, int *sd) const override {
        const int W = prm_.w, H = prm_.h;
        *w = W;
        *h = H;
        *sd = 0;
        const int fe = sizeof(F) == 8 ? IFL_DT_F64 : IFL_DT_F32;
        if (field >= IFL_F_R && field <= IFL_F_VDENS) {
            *elem = fe;
            *sd = field <= IFL_F_APLUSY ? 1 : 0;
            switch (field) {
            case IFL_F_R: *ptr = S_.r; *elem = IFL_DT_F64; return 0;
            case IFL_F_P: *ptr = S_.p; *elem = IFL_DT_F64; return 0;
            case IFL_F_Z: *ptr = S_.z; return 0;
            case IFL_F_S: *ptr = S_.sa; return 0;
            case IFL_F_PRECON: *ptr = S_.pc; *elem = IFL_DT_F64; return 0;
            case IFL_F_ADIAG: *ptr = S_.adiag; return 0;
            case IFL_F_APLUSX: *ptr = S_.ax; return 0;
            case IFL_F_APLUSY: *ptr = S_.ay; return 0;
            case IFL_F_UDENS: *ptr = S_.udens; *w = W + 1; return 0;
            case IFL_F_VDENS: *ptr = S_.vdens; *h = H + 1; return 0;
            }
        }
        int q = field >> 8, a = field & 0xff;
        if (q < 0 || q > 3 || !present(q)) return IFL_ERR_ARG;
        const Quant<F> &Q = S_.q[q];
        *w = Q.w;
        *h = Q.h;
        switch (a) {
        case IFL_A_SRC: *ptr = Q.src; *elem = fe; return 0;
        case IFL_A_DST: *ptr = Q.dst; *elem = fe; return 0;
        case IFL_A_PHI: *ptr = Q.phi; *elem = IFL_DT_F64; *w = Q.w + 1; *h = Q.h + 1; break;
        case IFL_A_VOLUME: *ptr = Q.vol; *elem = IFL_DT_F64; break;
        case IFL_A_NORMALX: *ptr = Q.nx; *elem = IFL_DT_F64; break;
        case IFL_A_NORMALY: *ptr = Q.ny; *elem = IFL_DT_F64; break;
        case IFL_A_CELL: *ptr = Q.cell; *elem = IFL_DT_U8; break;
        case IFL_A_BODY: *ptr = Q.body; *elem = IFL_DT_U8; break;
        default: return IFL_ERR_ARG;
        }
        return *ptr ? 0 : IFL_ERR_ARG;
    }

    int flip(int q) override {
        if (q < 0 || q > 3 || !present(q)) return IFL_ERR_ARG;
        std::swap(S_.q[q].src, S_.q[q].dst);
        return IFL_OK;
    }

    int read_pcg(ifl_step_stats *st) override {
        PcgOut o[2];
        unsigned fl = 0;
        if (check(cudaMemcpyAsync(o, scratch_.out, sizeof o, cudaMemcpyDeviceToHost, stream_), "stats") ||
            check(cudaMemcpyAsync(&fl, S_.flags, 4, cudaMemcpyDeviceToHost, stream_), "flags") ||
            check(cudaStreamSynchronize(stream_), "stats sync"))
            return IFL_ERR_CUDA;
        st->pressure = {o[0].iterations, o[0].status, o[0].max_error};
        st->heat = {o[1].iterations, o[1].status, o[1].max_error};
        st->device_flags = fl;
        st->steps = steps_;
        return IFL_OK;
    }

    int read_iteration_total(long long *out) override {
        unsigned long long v = 0;
        if (check(cudaMemcpyAsync(&v, scratch_.iter_total, 8, cudaMemcpyDeviceToHost, stream_), "iter total") ||
            check(cudaMemsetAsync(scratch_.iter_total, 0, 8, stream_), "iter reset") ||
            check(cudaStreamSynchronize(stream_), "iter sync"))
            return IFL_ERR_CUDA;
        *out = (long long)v;
        return IFL_OK;
    }

    size_t pitch() const override { return (size_t)P_; }
    size_t device_bytes() const override { return arena_bytes_; }
    int render(int heat, void *rgba, size_t bytes, bool on_device) override {
        const bool wide = heat && prm_.variant >= IFL_HEAT;
        const size_t need = (size_t)(wide ? 2 : 1) * prm_.w * prm_.h * 4;
        if (!rgba || bytes < need) return IFL_ERR_ARG;
        unsigned char *dst = (unsigned char *)rgba;
        if (!on_device) {
            if (image_bytes_ < need) {
                if (image_) cudaFree(image_);
                image_ = nullptr;
                image_bytes_ = 0;
                if (check(cudaMalloc(&image_, need), "image buffer")) return IFL_ERR_NOMEM;
                image_bytes_ = need;
            }
            dst = image_;
        }
        launch_render<F>(S_, dst, wide ? 1 : 0, stream_);
        launches_++;
        if (int e = launch_check("render")) return e;
        if (!on_device &&
            (check(cudaMemcpyAsync(rgba, image_, need, cudaMemcpyDeviceToHost, stream_), "image readback") ||
             check(cudaStreamSynchronize(stream_), "image sync")))
            return IFL_ERR_CUDA;
        return IFL_OK;
    }

    // ------------------------------------------------------ FLIP particles
    int particle_count(int *n) override {
        if (prm_.variant != IFL_FLIP || !n) return IFL_ERR_ARG;
        if (check(cudaMemcpyAsync(n, X_.ctl + FC_COUNT, sizeof(int), cudaMemcpyDeviceToHost, stream_), "count") ||
            check(cudaStreamSynchronize(stream_), "count sync"))
            return IFL_ERR_CUDA;
        return IFL_OK;
    }
    int read_particles(int which, double *out, int capacity, int *n) override {
        if (prm_.variant != IFL_FLIP || which < 0 || which > 5 || !out || !n) return IFL_ERR_ARG;
        if (int e = particle_count(n)) return e;
        if (*n > capacity) return IFL_ERR_ARG;
        if (check(cudaMemcpyAsync(out, particle_array(which), sizeof(double) * *n, cudaMemcpyDeviceToHost, stream_),
                  "particles") ||
            check(cudaStreamSynchronize(stream_), "particles sync"))
            return IFL_ERR_CUDA;
        return IFL_OK;
    }
    int write_particles(int which, const double *in, int n) override {
        if (prm_.variant != IFL_FLIP || which < 0 || which > 5 || !in || n < 0 || n > X_.cap) return IFL_ERR_ARG;
        if (check(cudaMemcpyAsync(particle_array(which), in, sizeof(double) * n, cudaMemcpyHostToDevice, stream_),
                  "particles") ||
            check(cudaStreamSynchronize(stream_), "particles sync"))
            return IFL_ERR_CUDA;
        return IFL_OK;
    }
    int set_particle_count(int n) override {
        if (prm_.variant != IFL_FLIP || n < 0 || n > X_.cap) return IFL_ERR_ARG;
        if (check(cudaMemcpyAsync(X_.ctl + FC_COUNT, &n, sizeof(int), cudaMemcpyHostToDevice, stream_), "count") ||
            check(cudaStreamSynchronize(stream_), "count sync"))
            return IFL_ERR_CUDA;
        flip_ready_ = true;  // the caller's particles replace the initial ones
        return IFL_OK;
    }
    int flip_init() override {
        if (prm_.variant != IFL_FLIP) return IFL_ERR_ARG;
        return flip_ensure_init();
    }
    int rng_state(uint32_t *get, const uint32_t *set) override {
        if (prm_.variant != IFL_FLIP) return IFL_ERR_ARG;
        if (set && check(cudaMemcpyAsync(X_.ctl + FC_RNG, set, 4, cudaMemcpyHostToDevice, stream_), "rng"))
            return IFL_ERR_CUDA;
        if (get && check(cudaMemcpyAsync(get, X_.ctl + FC_RNG, 4, cudaMemcpyDeviceToHost, stream_), "rng"))
            return IFL_ERR_CUDA;
        return check(cudaStreamSynchronize(stream_), "rng sync") ? IFL_ERR_CUDA : IFL_OK;
    }

    void *scene_ptr() override { return &S_; }
    void *scratch_ptr() override { return &scratch_; }
    bool has_quantity(int q) const override { return q >= 0 && q < 4 && present(q); }

  private:
    bool present(int q) const { return q != 1 || nq_ == 4; }

    double *particle_array(int which) const {
        return which == 0 ? X_.px : which == 1 ? X_.py : X_.prop[which - 2];
    }

    int flip_ensure_init() {
        if (flip_ready_) return IFL_OK;
        if constexpr (std::is_same<F, double>::value) {
            if (int e = upload_bodies()) return e;
            int t = tbegin(IFL_K_PARTICLES);
            launch_flip_init(S_, X_, stream_);
            tend(t);
            launches_ += 7;
            flip_ready_ = true;
            return launch_check("particle init");
        }
        return IFL_ERR_UNSUPPORTED;
    }

    // The FLIP phases (8-flip/Fluid.cpp:1356-1412); FP64 handles only.
    int flip_phase(int ph, double dt) {
        if constexpr (std::is_same<F, double>::value) {
            int t = -1;
            switch (ph) {
            case IFL_PH_P2G:
                if (int e = flip_ensure_init()) return e;
                t = tbegin(IFL_K_PARTICLES);
                launch_flip_p2g(S_, X_, stream_);
                launches_ += 25;
                break;
            case IFL_PH_FLIP_COPY:
                t = tbegin(IFL_K_FACES);
                launch_flip_copy(S_, stream_);
                launches_++;
                for (const auto &f : pending_) {
                    for (int q = 0; q < 4; q++) launch_inflow<F>(S_, q, f[0], f[1], f[0] + f[2], f[1] + f[3], f[4 + q], stream_);
                    launches_ += 4;
                }
                pending_.clear();
                break;
            case IFL_PH_G2P:
                t = tbegin(IFL_K_PARTICLES);
                launch_flip_g2p(S_, X_, stream_);
                launches_ += 2;
                break;
            case IFL_PH_PADVECT:
                t = tbegin(IFL_K_PARTICLES);
                launch_flip_advect(S_, X_, dt, stream_);
                launches_++;
                break;
            default: return IFL_ERR_ARG;
            }
            tend(t);
            return launch_check("flip phase");
        }
        (void)ph; (void)dt;
        return IFL_ERR_UNSUPPORTED;
    }

    void carve(char *base, Carver &c) {
        const size_t N = (size_t)P_ * rows_;
        const bool geo = prm_.variant >= IFL_SOLID;
        S_.sd = SDIdx::make(prm_.w, prm_.h);
        const size_t NS = S_.sd.total();
        S_.variant = prm_.variant;
        S_.w = prm_.w;
        S_.h = prm_.h;
        S_.P = P_;
        S_.nq = nq_;
        S_.hx = 1.0 / std::min(prm_.w, prm_.h);
        S_.rho_air = prm_.density_air;
        S_.rho_soot = prm_.density_soot;
        S_.diffusion = prm_.diffusion;
        S_.t_amb = 294.0;  // 7-variable-density/Fluid.cpp:950
        S_.g = 9.81;
        const double ox[4] = {0.5, 0.5, 0.0, 0.5}, oy[4] = {0.5, 0.5, 0.5, 0.0};
        const int qw[4] = {prm_.w, prm_.w, prm_.w + 1, prm_.w};
        const int qh[4] = {prm_.h, prm_.h, prm_.h, prm_.h + 1};
        for (int q = 0; q < 4; q++) {
            Quant<F> &Q = S_.q[q];
            Q = Quant<F>{};
            Q.w = qw[q];
            Q.h = qh[q];
            Q.ox = ox[q];
            Q.oy = oy[q];
            if (!present(q)) continue;
            Q.src = c.take<F>(base, N);
            Q.dst = c.take<F>(base, N);
            Q.cell = c.take<uint8_t>(base, N);
            if (geo) {
                Q.phi = prm_.variant >= IFL_CURVED ? c.take<double>(base, N) : nullptr;
                Q.vol = prm_.variant >= IFL_CURVED ? c.take<double>(base, N) : nullptr;
                Q.nx = c.take<double>(base, N);
                Q.ny = c.take<double>(base, N);
                Q.body = c.take<uint8_t>(base, N);
                Q.ready = c.take<uint8_t>(base, N);
                Q.list = c.take<int>(base, 2 * N);
            }
        }
        S_.r = c.take<double>(base, NS);
        S_.p = c.take<double>(base, NS);
        S_.z = c.take<F>(base, NS);
        S_.sa = c.take<F>(base, NS);
        S_.sb = c.take<F>(base, NS);
        S_.as = c.take<double>(base, NS);
        if (sizeof(F) == 8) S_.rf = (F *)S_.r;
        else S_.rf = c.take<F>(base, NS);
        S_.adiag = c.take<F>(base, NS);
        S_.ax = c.take<F>(base, NS);
        S_.ay = c.take<F>(base, NS);
        S_.mic = c.take<F>(base, 4 * NS);
        S_.pc = c.take<double>(base, NS);
        S_.nb = c.take<uint8_t>(base, NS);
        if (prm_.variant >= IFL_VARDENS) {
            S_.udens = c.take<F>(base, N);
            S_.vdens = c.take<F>(base, N);
        } else {
            S_.udens = S_.vdens = nullptr;
        }
        d_bodies_ = c.take<DevBody>(base, 256);
        S_.bodies = d_bodies_;
        S_.nbodies = 0;
        S_.flags = c.take<unsigned>(base, 8);
        M_ = PcgF32{};
        f32_solves_ = prm_.variant == IFL_FLIP && prm_.precision == IFL_FP32;
        if (f32_solves_) {  // FP32-form solves beside the FP64 fields and particles
            M_.adiag = c.take<float>(base, NS);
            M_.ax = c.take<float>(base, NS);
            M_.ay = c.take<float>(base, NS);
            M_.mic = c.take<float>(base, 4 * NS);
            M_.rf = c.take<float>(base, NS);
            M_.z = c.take<float>(base, NS);
            M_.sa = c.take<float>(base, NS);
            M_.sb = c.take<float>(base, NS);
        }
        X_ = FlipState{};
        if (prm_.variant == IFL_FLIP) {
            const int w = prm_.w, h = prm_.h, cells = w * h;
            X_.cap = 12 * cells;  // _maxParticles = w*h*_MaxPerCell
            X_.px = c.take<double>(base, X_.cap);
            X_.py = c.take<double>(base, X_.cap);
            for (int k = 0; k < 4; k++) X_.prop[k] = c.take<double>(base, X_.cap);
            X_.node_off[0] = 0;
            X_.node_off[1] = cells;
            X_.node_off[2] = cells + (w + 1) * h;
            X_.node_off[3] = X_.node_off[2] + w * (h + 1);
            const int nodes = X_.node_off[3];
            X_.bcount = c.take<unsigned long long>(base, nodes);
            X_.bstart = c.take<unsigned long long>(base, nodes + 1);
            X_.brank = c.take<int>(base, 3 * (size_t)X_.cap);
            X_.blist = c.take<int>(base, 3 * (size_t)X_.cap);
            X_.cell_count = c.take<int>(base, cells);
            X_.seedv = c.take<unsigned long long>(base, cells);
            X_.seedx = c.take<unsigned long long>(base, cells + 1);
            X_.scan_tmp = c.take<unsigned long long>(base, flip_scan_tiles(std::max(nodes, cells)));
            X_.cand = c.take<int>(base, X_.cap);
            X_.ctl = c.take<int>(base, FC_WORDS);
        }
        scratch_.max_blocks = max_blocks_;
        scratch_.partials = c.take<double>(base, 4 * pcg_chunks(S_.sd));
        scratch_.barrier = c.take<unsigned>(base, 2);
        scratch_.halo = c.take<unsigned long long>(base, 2 * (size_t)S_.sd.S * S_.sd.D);
        scratch_.out = c.take<PcgOut>(base, 2);
        scratch_.iter_total = c.take<unsigned long long>(base, 1);
    }

    int upload_bodies() {
        if (!bodies_dirty_) return IFL_OK;
        if (!staging_) {
            if (check(cudaMallocHost((void **)&staging_, 256 * sizeof(DevBody)), "pinned staging") ||
                check(cudaEventCreateWithFlags(&staging_done_, cudaEventDisableTiming), "staging event"))
                return IFL_ERR_CUDA;
        } else if (check(cudaEventSynchronize(staging_done_), "staging wait")) {
            return IFL_ERR_CUDA;  // the previous upload must have left the buffer
        }
        DevBody *db = staging_;
        for (size_t i = 0; i < bodies_.size(); i++) to_dev_body(bodies_[i], db[i]);
        if (check(cudaMemcpyAsync(d_bodies_, db, bodies_.size() * sizeof(DevBody), cudaMemcpyHostToDevice,
                                  stream_),
                  "bodies") ||
            check(cudaEventRecord(staging_done_, stream_), "staging record"))
            return IFL_ERR_CUDA;
        S_.nbodies = (int)bodies_.size();
        bodies_dirty_ = false;
        return IFL_OK;
    }

    void assemble(double dt, int what) {
        int t = tbegin(IFL_K_ASSEMBLE);
        launch_assemble<F>(S_, dt, what, stream_);
        tend(t);
        launches_++;
    }

    void extrapolate(unsigned qmask) {
        if (prm_.variant < IFL_SOLID) return;
        int t = tbegin(IFL_K_EXTRAPOLATE);
        launch_extrapolate<F>(S_, qmask, stream_);
        tend(t);
        launches_ += 2;
    }

    int pcg(int mode, bool heat) {
        PcgConfig cfg;
        cfg.mode = mode;
        cfg.limit = heat ? prm_.max_iter_heat : prm_.max_iter_pressure;
        cfg.pinned = heat ? pinned_heat_ : pinned_;
        cfg.heat = heat ? 1 : 0;
        cfg.wait_limit = wait_limit_;
        int G = 0;
        int t = tbegin(IFL_K_PCG);
        cudaError_t e;
        if constexpr (std::is_same<F, double>::value) {
            e = f32_solves_ ? launch_pcg_f32(S_, M_, scratch_, cfg, stream_, &G)
                            : launch_pcg<F>(S_, scratch_, cfg, stream_, &G);
        } else {
            e = launch_pcg<F>(S_, scratch_, cfg, stream_, &G);
        }
        tend(t);
        if (check(e, "pcg launch")) return IFL_ERR_CUDA;
        launches_++;
        return IFL_OK;
    }

    // project() of steps 1-2: Gauss-Seidel sweeps on p, which persists between steps.
    int gauss_seidel(double dt) {
        int t = tbegin(IFL_K_PCG);
        cudaError_t e = launch_gs<F>(S_, scratch_, dt, prm_.max_iter_pressure, pinned_, stream_, wait_limit_);
        tend(t);
        if (check(e, "gauss-seidel launch")) return IFL_ERR_CUDA;
        launches_++;
        return IFL_OK;
    }

    // r = T; heat matrix; MIC(0); PCG; T = p  (7-variable-density/Fluid.cpp:1001-1005)
    int heat_solve(double dt) {
        int t = tbegin(IFL_K_ASSEMBLE);
        launch_heat_assemble<F>(S_, dt, stream_);
        tend(t);
        launches_++;
        if (int e = pcg(PCG_FACTOR | PCG_SOLVE, true)) return e;
        t = tbegin(IFL_K_ASSEMBLE);
        launch_sd_to_rows<F>(S_, S_.q[1].src, S_.p, stream_);
        tend(t);
        launches_++;
        return launch_check("T = p");
    }

    int launch_check(const char *what) {
        return check(cudaGetLastError(), what) ? IFL_ERR_CUDA : IFL_OK;
    }

    void release() {
        if (stream_) cudaStreamSynchronize(stream_);
        release_timing();
        if (staging_) cudaFreeHost(staging_);
        staging_ = nullptr;
        if (staging_done_) cudaEventDestroy(staging_done_);
        staging_done_ = nullptr;
        if (arena_) cudaFree(arena_);
        arena_ = nullptr;
        if (image_) cudaFree(image_);
        image_ = nullptr;
        if (own_stream_ && stream_) cudaStreamDestroy(stream_);
        stream_ = nullptr;
    }

    Scene<F> S_{};
    PcgF32 M_{};
    bool f32_solves_ = false;  // step 8 with IFL_FP32: FP32-form PCG, FP64 everything else
    FlipState X_{};
    bool flip_ready_ = false;
    std::vector<std::array<double, 8>> pending_;  // FLIP inflows of the next update
    PcgScratch scratch_{};
    DevBody *d_bodies_ = nullptr;
    DevBody *staging_ = nullptr;  // pinned host copy of the body table
    cudaEvent_t staging_done_ = nullptr;
    void *arena_ = nullptr;
    size_t arena_bytes_ = 0;
    unsigned char *image_ = nullptr;  // device staging of toImage for host readback
    size_t image_bytes_ = 0;
    int P_ = 0, rows_ = 0, nq_ = 3, max_blocks_ = 1;
};

void to_dev_body(const ifl_body &b, DevBody &d) {
    d.type = b.type;
    d.pad_ = 0;
    d.px = b.pos_x;
    d.py = b.pos_y;
    d.sx = b.scale_x;
    d.sy = b.type == 0 ? b.scale_y : b.scale_x;  // SolidSphere(x, y, s, ...) sets both scales to s
    d.vx = b.vel_x;
    d.vy = b.vel_y;
    d.vth = b.vel_theta;
    d.cpos = std::cos(b.theta);
    d.spos = std::sin(b.theta);
    d.cneg = std::cos(-b.theta);
    d.sneg = std::sin(-b.theta);
}

// ------------------------------------------------------------ SolverBase
int SolverBase::tbegin(int group) {
    if (!timing_on_ || recs_.size() >= 1u << 16) return -1;
    TimedRec r;
    r.group = group;
    for (cudaEvent_t *ev : {&r.start, &r.stop}) {
        if (!event_pool_.empty()) {
            *ev = event_pool_.back();
            event_pool_.pop_back();
        } else if (cudaEventCreate(ev) != cudaSuccess) {
            return -1;
        }
    }
    cudaEventRecord(r.start, stream_);
    recs_.push_back(r);
    return (int)recs_.size() - 1;
}

void SolverBase::tend(int rec) {
    if (rec >= 0) cudaEventRecord(recs_[rec].stop, stream_);
}

int SolverBase::set_timing(bool on) {
    timing_on_ = on;
    return IFL_OK;
}

int SolverBase::get_timing(ifl_timing *out) {
    std::memset(out, 0, sizeof *out);
    if (check(cudaStreamSynchronize(stream_), "timing sync")) return IFL_ERR_CUDA;
    for (TimedRec &r : recs_) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, r.start, r.stop) == cudaSuccess) {
            out->ms[r.group] += ms;
            out->launches[r.group]++;
        }
        event_pool_.push_back(r.start);
        event_pool_.push_back(r.stop);
    }
    recs_.clear();
    long long it = 0;
    if (int e = read_iteration_total(&it)) return e;
    out->pcg_iterations = it;
    return IFL_OK;
}

void SolverBase::release_timing() {
    for (TimedRec &r : recs_) {
        event_pool_.push_back(r.start);
        event_pool_.push_back(r.stop);
    }
    recs_.clear();
    for (cudaEvent_t e : event_pool_) cudaEventDestroy(e);
    event_pool_.clear();
}

bool SolverBase::check(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return false;
    err_ = std::string(what) + ": " + cudaGetErrorString(e);
    return true;
}

int SolverBase::set_bodies(const ifl_body *b, int n) {
    if (n < 0 || n > 256 || (n > 0 && !b)) return IFL_ERR_ARG;
    for (int i = 0; i < n; i++)
        if (b[i].type != 0 && b[i].type != 1) return IFL_ERR_ARG;
    bodies_.assign(b, b + n);
    bodies_dirty_ = true;
    return IFL_OK;
}

// SolidBody::update (4-solid-boundaries/Fluid.cpp:140-148)
int SolverBase::advance_bodies(double dt) {
    for (ifl_body &b : bodies_) {
        b.pos_x += b.vel_x * dt;
        b.pos_y += b.vel_y * dt;
        b.theta += b.vel_theta * dt;
    }
    bodies_dirty_ = true;
    return IFL_OK;
}

namespace {
// Dense row-major <-> strip-diagonal permutation on the host (field transfer only).
void sd_gather(const SDIdx &sd, const char *sdbuf, char *dense, size_t es) {
    for (int y = 0; y < sd.H; y++)
        for (int x = 0; x < sd.W; x++)
            std::memcpy(dense + ((size_t)x + (size_t)y * sd.W) * es, sdbuf + sd.slot(x, y) * es, es);
}
void sd_scatter(const SDIdx &sd, const char *dense, char *sdbuf, size_t es) {
    for (int y = 0; y < sd.H; y++)
        for (int x = 0; x < sd.W; x++)
            std::memcpy(sdbuf + sd.slot(x, y) * es, dense + ((size_t)x + (size_t)y * sd.W) * es, es);
}
}  // namespace

int SolverBase::read_field(int field, void *host, size_t bytes, int dtype) {
    void *ptr;
    int elem, w, h, sdl;
    if (int e = field_info(field, &ptr, &elem, &w, &h, &sdl)) return e;
    const size_t n = (size_t)w * h;
    const size_t out_es = dtype == IFL_DT_F64 ? 8 : dtype == IFL_DT_F32 ? 4 : dtype == IFL_DT_U8 ? 1 : 0;
    if (!out_es || !host || bytes < n * out_es) return IFL_ERR_ARG;
    if ((elem == IFL_DT_U8) != (dtype == IFL_DT_U8)) return IFL_ERR_ARG;
    const size_t es = elem == IFL_DT_F64 ? 8 : elem == IFL_DT_F32 ? 4 : 1;
    std::vector<char> tmp;
    void *dst = host;
    if (elem != dtype || sdl) {
        tmp.resize(n * es);
        dst = tmp.data();
    }
    if (sdl) {
        const SDIdx sd = sd_index();
        std::vector<char> raw(sd.total() * es);
        if (check(cudaMemcpyAsync(raw.data(), ptr, raw.size(), cudaMemcpyDeviceToHost, stream()), "read field") ||
            check(cudaStreamSynchronize(stream()), "read sync"))
            return IFL_ERR_CUDA;
        sd_gather(sd, raw.data(), (char *)dst, es);
        if (elem == dtype) std::memcpy(host, dst, n * es);
    } else if (check(cudaMemcpy2DAsync(dst, w * es, ptr, pitch() * es, w * es, h, cudaMemcpyDeviceToHost,
                                       stream()),
                     "read field") ||
               check(cudaStreamSynchronize(stream()), "read sync")) {
        return IFL_ERR_CUDA;
    }
    if (elem != dtype) {
        if (elem == IFL_DT_F64) {
            const double *s = (const double *)dst;
            float *o = (float *)host;
            for (size_t i = 0; i < n; i++) o[i] = (float)s[i];
        } else {
            const float *s = (const float *)dst;
            double *o = (double *)host;
            for (size_t i = 0; i < n; i++) o[i] = (double)s[i];
        }
    }
    return IFL_OK;
}

int SolverBase::write_field(int field, const void *host, size_t bytes, int dtype) {
    void *ptr;
    int elem, w, h, sdl;
    if (int e = field_info(field, &ptr, &elem, &w, &h, &sdl)) return e;
    const size_t n = (size_t)w * h;
    const size_t in_es = dtype == IFL_DT_F64 ? 8 : dtype == IFL_DT_F32 ? 4 : dtype == IFL_DT_U8 ? 1 : 0;
    if (!in_es || !host || bytes < n * in_es) return IFL_ERR_ARG;
    if ((elem == IFL_DT_U8) != (dtype == IFL_DT_U8)) return IFL_ERR_ARG;
    const size_t es = elem == IFL_DT_F64 ? 8 : elem == IFL_DT_F32 ? 4 : 1;
    std::vector<char> tmp;
    const void *src = host;
    if (elem != dtype) {
        tmp.resize(n * es);
        if (elem == IFL_DT_F64) {
            const float *s = (const float *)host;
            double *o = (double *)tmp.data();
            for (size_t i = 0; i < n; i++) o[i] = (double)s[i];
        } else {
            const double *s = (const double *)host;
            float *o = (float *)tmp.data();
            for (size_t i = 0; i < n; i++) o[i] = (float)s[i];
        }
        src = tmp.data();
    }
    if (sdl) {
        const SDIdx sd = sd_index();
        std::vector<char> raw(sd.total() * es, 0);
        sd_scatter(sd, (const char *)src, raw.data(), es);
        if (check(cudaMemcpyAsync(ptr, raw.data(), raw.size(), cudaMemcpyHostToDevice, stream()), "write field") ||
            check(cudaStreamSynchronize(stream()), "write sync"))
            return IFL_ERR_CUDA;
        return IFL_OK;
    }
    if (check(cudaMemcpy2DAsync(ptr, pitch() * es, src, w * es, w * es, h, cudaMemcpyHostToDevice, stream()),
              "write field") ||
        check(cudaStreamSynchronize(stream()), "write sync"))
        return IFL_ERR_CUDA;
    return IFL_OK;
}

// Step 8 keeps FP64 fields and particles in both forms; IFL_FP32 selects its
// FP32-form solves only.
size_t solver_device_bytes(const ifl_params &p, int max_blocks) {
    if (p.precision == IFL_FP32 && p.variant != IFL_FLIP) return SolverImpl<float>::arena_size(p, max_blocks);
    return SolverImpl<double>::arena_size(p, max_blocks);
}

std::unique_ptr<SolverBase> make_solver(const ifl_params &p) {
    if (p.precision == IFL_FP32 && p.variant != IFL_FLIP) return std::unique_ptr<SolverBase>(new SolverImpl<float>(p));
    return std::unique_ptr<SolverBase>(new SolverImpl<double>(p));
}

}  // namespace ifl
