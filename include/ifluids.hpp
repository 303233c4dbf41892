// ifluids.hpp - header-only C++ drop-in for the reference's FluidSolver surface.
//
// Mirrors the classes a program written against tunabrain/incremental-fluids
// uses (3-conjugate-gradients/Fluid.cpp:401-453, 4-solid-boundaries/Fluid.cpp:79-241
// and :836-901, 7-variable-density/Fluid.cpp:945-1045): construct a FluidSolver,
// call addInflow and update(dt) every step, move the bodies with
// SolidBody::update between steps.  Everything runs on the GPU through the C
// ABI of ifluids.h; fields come back with read() (the reference only had
// toImage).  Errors become std::runtime_error.
#pragma once
#include <stdexcept>
#include <string>
#include <vector>

#include "ifluids.h"

namespace ifluids {

// SolidBody / SolidBox / SolidSphere: same parameters and Euler update as the
// reference (4-solid-boundaries/Fluid.cpp:109-148, 155-156, 207-208).
class SolidBody {
  public:
    virtual ~SolidBody() = default;
    void update(double timestep) {
        b_.pos_x += b_.vel_x * timestep;
        b_.pos_y += b_.vel_y * timestep;
        b_.theta += b_.vel_theta * timestep;
    }
    const ifl_body &state() const { return b_; }

  protected:
    SolidBody(int type, double x, double y, double sx, double sy, double t, double vx, double vy, double vt) {
        b_.type = type;
        b_.pad_ = 0;
        b_.pos_x = x;
        b_.pos_y = y;
        b_.scale_x = sx;
        b_.scale_y = sy;
        b_.theta = t;
        b_.vel_x = vx;
        b_.vel_y = vy;
        b_.vel_theta = vt;
    }
    ifl_body b_;
};

class SolidBox : public SolidBody {
  public:
    SolidBox(double x, double y, double sx, double sy, double t, double vx, double vy, double vt)
        : SolidBody(0, x, y, sx, sy, t, vx, vy, vt) {}
};

class SolidSphere : public SolidBody {
  public:
    SolidSphere(double x, double y, double s, double t, double vx, double vy, double vt)
        : SolidBody(1, x, y, s, s, t, vx, vy, vt) {}
};

class FluidSolver {
  public:
    // 3-conjugate-gradients (variant = IFL_GS_EULER / IFL_GS for 1-matrixless /
    // 2-better-advection, the same constructor in the reference)
    FluidSolver(int w, int h, double density, int precision = IFL_FP64, int variant = IFL_PLAIN) {
        init(variant, w, h, density, 1.0, 0.01, precision);
    }
    // 4-solid-boundaries (variant = IFL_CURVED for 5-curved-boundaries)
    FluidSolver(int w, int h, double density, const std::vector<const SolidBody *> &bodies,
                int variant = IFL_SOLID, int precision = IFL_FP64)
        : bodies_(&bodies) {
        init(variant, w, h, density, 1.0, 0.01, precision);
    }
    // 7-variable-density (variant = IFL_HEAT for 6-heat, IFL_FLIP for 8-flip)
    FluidSolver(int w, int h, double rhoAir, double rhoSoot, double diffusion,
                const std::vector<const SolidBody *> &bodies, int variant = IFL_VARDENS,
                int precision = IFL_FP64)
        : bodies_(&bodies) {
        init(variant, w, h, rhoAir, rhoSoot, diffusion, precision);
    }
    ~FluidSolver() {
        if (h_) ifl_destroy(h_);
    }
    FluidSolver(const FluidSolver &) = delete;
    FluidSolver &operator=(const FluidSolver &) = delete;

    void addInflow(double x, double y, double w, double h, double d, double u, double v) {
        check(ifl_add_inflow(h_, x, y, w, h, d, 0.0, u, v), "addInflow");
    }
    void addInflow(double x, double y, double w, double h, double d, double t, double u, double v) {
        check(ifl_add_inflow(h_, x, y, w, h, d, t, u, v), "addInflow");
    }
    // The bodies are held by reference, as in the reference: their current
    // state is sent to the device at every update.  Step 8's update() adds
    // its own inflow after copy() (8-flip/Fluid.cpp:1368); so does this one
    // unless builtinInflow(false) was called.
    void update(double timestep) {
        if (variant_ == IFL_FLIP && builtin_inflow_)
            check(ifl_add_inflow(h_, 0.45, 0.2, 0.2, 0.05, 1.0, ambientT(), 0.0, 0.0), "addInflow");
        if (bodies_) {
            std::vector<ifl_body> tab;
            tab.reserve(bodies_->size());
            for (const SolidBody *b : *bodies_) tab.push_back(b->state());
            check(ifl_set_bodies(h_, tab.data(), (int)tab.size()), "set bodies");
        }
        check(ifl_update(h_, timestep), "update");
    }
    double ambientT() const { return ifl_ambient_t(h_); }

    // Field readback: quantity field (IFL_FIELD(IFL_Q_D, IFL_A_SRC), ...) or
    // solver array (IFL_F_P, ...) as a dense row-major FP64 vector.
    std::vector<double> read(int field, int *w = nullptr, int *h = nullptr) {
        int fw = 0, fh = 0;
        check(ifl_field_shape(h_, field, &fw, &fh), "field shape");
        std::vector<double> out((size_t)fw * fh);
        check(ifl_read_field(h_, field, out.data(), out.size() * sizeof(double), IFL_DT_F64), "read field");
        if (w) *w = fw;
        if (h) *h = fh;
        return out;
    }
    // Step 8: particle positions or carried values (IFL_P_X .. IFL_P_V).
    std::vector<double> particles(int which) {
        int n = 0;
        check(ifl_particle_count(h_, &n), "particle count");
        std::vector<double> out((size_t)n);
        check(ifl_read_particles(h_, which, out.data(), n, &n), "particles");
        return out;
    }
    void builtinInflow(bool on) { builtin_inflow_ = on; }
    // FluidSolver::toImage: rgba holds w*h*4 bytes (2*w*h*4 with renderHeat in steps 6-8).
    void toImage(unsigned char *rgba, bool renderHeat = false) {
        int w = 0, h = 0;
        check(ifl_field_shape(h_, IFL_FIELD(IFL_Q_D, IFL_A_SRC), &w, &h), "field shape");
        const bool wide = renderHeat && variant_ >= IFL_HEAT;
        check(ifl_render(h_, renderHeat ? 1 : 0, rgba, (size_t)(wide ? 2 : 1) * w * h * 4, 0), "toImage");
    }
    ifl_step_stats stats() {
        ifl_step_stats st;
        check(ifl_get_stats(h_, &st), "stats");
        return st;
    }
    ifl_solver *handle() { return h_; }

  private:
    void init(int variant, int w, int h, double ra, double rs, double diff, int precision) {
        ifl_params p;
        ifl_default_params(&p, variant, w, h);
        p.density_air = ra;
        p.density_soot = rs;
        p.diffusion = diff;
        p.precision = precision;
        variant_ = variant;
        check(ifl_create(&p, &h_), "create");
    }
    void check(int rc, const char *what) {
        if (rc != IFL_OK)
            throw std::runtime_error(std::string("ifluids: ") + what + " failed (" + std::to_string(rc) +
                                     "): " + (h_ ? ifl_last_error(h_) : ""));
    }
    ifl_solver *h_ = nullptr;
    int variant_ = IFL_PLAIN;
    bool builtin_inflow_ = true;
    const std::vector<const SolidBody *> *bodies_ = nullptr;
};

}  // namespace ifluids
