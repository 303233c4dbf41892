// capi.cpp - the extern "C" entry points declared in include/ifluids.h.
// Each one validates its arguments, forwards to the solver object and turns
// every failure into a status code; no exception crosses the ABI.
#include <cstring>
#include <new>

#include "solver.h"

struct ifl_solver {
    std::unique_ptr<ifl::SolverBase> impl;
};

namespace {
template <typename Fn>
int guarded(ifl_solver *s, Fn fn) {
    if (!s || !s->impl) return IFL_ERR_ARG;
    if (s->impl->activate() != 0) {
        s->impl->set_error("cannot make the handle's device current");
        return IFL_ERR_CUDA;
    }
    try {
        return fn(*s->impl);
    } catch (const std::bad_alloc &) {
        s->impl->set_error("host allocation failed");
        return IFL_ERR_NOMEM;
    } catch (...) {
        s->impl->set_error("internal error");
        return IFL_ERR_ARG;
    }
}
}  // namespace

extern "C" {

void ifl_default_params(ifl_params *p, int variant, int w, int h) {
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    p->variant = variant;
    p->w = w;
    p->h = h;
    p->precision = IFL_FP64;
    p->density_air = 0.1;   // every reference main(): density / densityAir = 0.1
    p->density_soot = 1.0;  // 7-variable-density/Fluid.cpp:1090
    p->diffusion = 0.01;    // 7-variable-density/Fluid.cpp:1091
    p->max_iter_pressure = variant == IFL_PLAIN ? 600 : 2000;  // 3-conjugate-gradients/Fluid.cpp:437
    p->max_iter_heat = 2000;                                    // 7-variable-density/Fluid.cpp:1004
    p->stream = nullptr;
}

int ifl_create(const ifl_params *p, ifl_solver **out) {
    if (!p || !out) return IFL_ERR_ARG;
    *out = nullptr;
    if (p->variant < IFL_PLAIN || p->variant > IFL_VARDENS) return IFL_ERR_ARG;
    if (p->w < 2 || p->h < 2 || p->w > 32768 || p->h > 32768) return IFL_ERR_ARG;
    if (p->precision != IFL_FP64 && p->precision != IFL_FP32) return IFL_ERR_ARG;
    if (p->device < 0) return IFL_ERR_ARG;
    if (p->max_iter_pressure < 0 || p->max_iter_heat < 0) return IFL_ERR_ARG;
    if (!(p->density_air > 0.0)) return IFL_ERR_ARG;
    ifl_solver *s = new (std::nothrow) ifl_solver;
    if (!s) return IFL_ERR_NOMEM;
    try {
        s->impl = ifl::make_solver(*p);
    } catch (...) {
        delete s;
        return IFL_ERR_NOMEM;
    }
    int e = s->impl->init();
    if (e != IFL_OK) {
        delete s;
        return e;
    }
    *out = s;
    return IFL_OK;
}

int ifl_destroy(ifl_solver *s) {
    if (!s) return IFL_ERR_ARG;
    if (s->impl) s->impl->activate();
    delete s;
    return IFL_OK;
}

int ifl_set_bodies(ifl_solver *s, const ifl_body *bodies, int n) {
    return guarded(s, [&](ifl::SolverBase &v) { return v.set_bodies(bodies, n); });
}

int ifl_get_bodies(ifl_solver *s, ifl_body *bodies, int capacity, int *n) {
    return guarded(s, [&](ifl::SolverBase &v) {
        const auto &b = v.bodies();
        if (n) *n = (int)b.size();
        if (capacity < (int)b.size() || (!bodies && !b.empty())) return (int)IFL_ERR_ARG;
        for (size_t i = 0; i < b.size(); i++) bodies[i] = b[i];
        return (int)IFL_OK;
    });
}

int ifl_advance_bodies(ifl_solver *s, double dt) {
    return guarded(s, [&](ifl::SolverBase &v) { return v.advance_bodies(dt); });
}

int ifl_add_inflow(ifl_solver *s, double x, double y, double w, double h, double d, double t, double u,
                   double v) {
    return guarded(s, [&](ifl::SolverBase &m) { return m.add_inflow(x, y, w, h, d, t, u, v); });
}

int ifl_update(ifl_solver *s, double dt) {
    return guarded(s, [&](ifl::SolverBase &v) { return v.update(dt); });
}

int ifl_run_phase(ifl_solver *s, int phase, double dt) {
    return guarded(s, [&](ifl::SolverBase &v) { return v.run_phase(phase, dt); });
}

double ifl_ambient_t(const ifl_solver *s) {
    (void)s;
    return 294.0;  // 7-variable-density/Fluid.cpp:950
}

int ifl_field_shape(const ifl_solver *s, int field, int *w, int *h) {
    if (!s || !s->impl || !w || !h) return IFL_ERR_ARG;
    void *p;
    int elem, sd;
    return s->impl->field_info(field, &p, &elem, w, h, &sd);
}

int ifl_read_field(ifl_solver *s, int field, void *host, size_t bytes, int dtype) {
    return guarded(s, [&](ifl::SolverBase &v) { return v.read_field(field, host, bytes, dtype); });
}

int ifl_write_field(ifl_solver *s, int field, const void *host, size_t bytes, int dtype) {
    return guarded(s, [&](ifl::SolverBase &v) { return v.write_field(field, host, bytes, dtype); });
}

int ifl_flip(ifl_solver *s, int quantity) {
    return guarded(s, [&](ifl::SolverBase &v) { return v.flip(quantity); });
}

int ifl_get_stats(ifl_solver *s, ifl_step_stats *out) {
    if (!out) return IFL_ERR_ARG;
    return guarded(s, [&](ifl::SolverBase &v) {
        int e = v.read_pcg(out);
        if (e == IFL_OK && (out->device_flags & ifl::FLAG_TIMEOUT)) {
            v.set_error("a bounded device-side wait timed out");
            return (int)IFL_ERR_TIMEOUT;
        }
        return e;
    });
}

int ifl_set_pinned_iterations(ifl_solver *s, int pressure, int heat) {
    return guarded(s, [&](ifl::SolverBase &v) {
        v.set_pinned(pressure < 0 ? -1 : pressure, heat < 0 ? -1 : heat);
        return (int)IFL_OK;
    });
}

int ifl_set_timing(ifl_solver *s, int on) {
    return guarded(s, [&](ifl::SolverBase &v) { return v.set_timing(on != 0); });
}

int ifl_get_timing(ifl_solver *s, ifl_timing *out) {
    if (!out) return IFL_ERR_ARG;
    return guarded(s, [&](ifl::SolverBase &v) { return v.get_timing(out); });
}

int ifl_synchronize(ifl_solver *s) {
    return guarded(s, [&](ifl::SolverBase &v) {
        cudaError_t e = cudaStreamSynchronize(v.stream());
        if (e != cudaSuccess) {
            v.set_error(std::string("synchronize: ") + cudaGetErrorString(e));
            return (int)IFL_ERR_CUDA;
        }
        return (int)IFL_OK;
    });
}

void *ifl_stream(ifl_solver *s) { return (s && s->impl) ? (void *)s->impl->stream() : nullptr; }

int64_t ifl_launch_count(const ifl_solver *s) { return (s && s->impl) ? s->impl->launches() : 0; }

const char *ifl_last_error(const ifl_solver *s) {
    return (s && s->impl) ? s->impl->error().c_str() : "invalid handle";
}

const char *ifl_version(void) { return "ifluids-gb300 0.1 (sm_103a)"; }

}  // extern "C"
