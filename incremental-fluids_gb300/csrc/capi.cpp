// capi.cpp - the extern "C" entry points declared in include/ifluids.h.
// Each one validates its arguments, forwards to the solver object and turns
// every failure into a status code; no exception crosses the ABI.
#include <cstring>
#include <new>
#include <vector>

#include "solver.h"

struct ifl_solver {
    std::unique_ptr<ifl::SolverBase> impl;
};

struct ifl_batch {
    std::unique_ptr<ifl::BatchBase> impl;
};

struct ifl_server {
    ifl::Server *impl = nullptr;
    bool dry = false;
    ~ifl_server() { ifl::server_destroy(impl); }
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
thread_local std::string g_batch_create_error;

template <typename Fn>
int bguarded(ifl_batch *b, Fn fn) {
    if (!b || !b->impl) return IFL_ERR_ARG;
    if (cudaSetDevice(b->impl->device()) != cudaSuccess) {
        b->impl->set_error("cannot make the batch's device current");
        return IFL_ERR_CUDA;
    }
    try {
        return fn(*b->impl);
    } catch (const std::bad_alloc &) {
        b->impl->set_error("host allocation failed");
        return IFL_ERR_NOMEM;
    } catch (...) {
        b->impl->set_error("internal error");
        return IFL_ERR_ARG;
    }
}
}  // namespace

namespace {
template <typename Fn>
int sguarded(ifl_server *s, Fn fn) {
    if (!s || !s->impl) return IFL_ERR_ARG;
    if (!s->dry && cudaSetDevice(ifl::server_device(s->impl)) != cudaSuccess) {
        ifl::server_set_error(s->impl, "cannot make the server's device current");
        return IFL_ERR_CUDA;
    }
    try {
        return fn(s->impl);
    } catch (const std::bad_alloc &) {
        ifl::server_set_error(s->impl, "host allocation failed");
        return IFL_ERR_NOMEM;
    } catch (...) {
        ifl::server_set_error(s->impl, "internal error");
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
    p->max_iter_pressure = variant <= IFL_PLAIN ? 600 : 2000;  // 1-matrixless/Fluid.cpp:286, 3-conjugate-gradients/Fluid.cpp:437
    p->max_iter_heat = 2000;                                    // 7-variable-density/Fluid.cpp:1004
    p->stream = nullptr;
}

int ifl_create(const ifl_params *p, ifl_solver **out) {
    if (!p || !out) return IFL_ERR_ARG;
    *out = nullptr;
    if (p->variant < IFL_GS_EULER || p->variant > IFL_FLIP) return IFL_ERR_ARG;
    if (p->w < 2 || p->h < 2 || p->w > 32768 || p->h > 32768) return IFL_ERR_ARG;
    if (p->variant <= IFL_GS && p->h > ifl::gs_max_rows()) return IFL_ERR_UNSUPPORTED;  // one CTA of strips
    if (p->precision != IFL_FP64 && p->precision != IFL_FP32) return IFL_ERR_ARG;
    if (p->variant == IFL_FLIP && (int64_t)p->w * p->h * 12 > 0x7fffffff) return IFL_ERR_UNSUPPORTED;
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

int ifl_render(ifl_solver *s, int heat, void *rgba, size_t bytes, int on_device) {
    return guarded(s, [&](ifl::SolverBase &v) { return v.render(heat, rgba, bytes, on_device != 0); });
}

int ifl_flip(ifl_solver *s, int quantity) {
    return guarded(s, [&](ifl::SolverBase &v) { return v.flip(quantity); });
}

int ifl_flip_init(ifl_solver *s) {
    return guarded(s, [&](ifl::SolverBase &v) { return v.flip_init(); });
}

int ifl_particle_count(ifl_solver *s, int *n) {
    return guarded(s, [&](ifl::SolverBase &v) { return v.particle_count(n); });
}

int ifl_read_particles(ifl_solver *s, int which, double *out, int capacity, int *n) {
    return guarded(s, [&](ifl::SolverBase &v) { return v.read_particles(which, out, capacity, n); });
}

int ifl_write_particles(ifl_solver *s, int which, const double *in, int n) {
    return guarded(s, [&](ifl::SolverBase &v) { return v.write_particles(which, in, n); });
}

int ifl_set_particle_count(ifl_solver *s, int n) {
    return guarded(s, [&](ifl::SolverBase &v) { return v.set_particle_count(n); });
}

int ifl_get_rng_state(ifl_solver *s, uint32_t *state) {
    if (!state) return IFL_ERR_ARG;
    return guarded(s, [&](ifl::SolverBase &v) { return v.rng_state(state, nullptr); });
}

int ifl_set_rng_state(ifl_solver *s, uint32_t state) {
    return guarded(s, [&](ifl::SolverBase &v) { return v.rng_state(nullptr, &state); });
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

int ifl_set_wait_limit(ifl_solver *s, int64_t polls) {
    if (polls < 0) return IFL_ERR_ARG;
    return guarded(s, [&](ifl::SolverBase &v) {
        v.set_wait_limit((long long)polls);
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

// ------------------------------------------------------------------ serving
void ifl_server_default_params(ifl_server_params *p, int variant, int precision) {
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    p->variant = variant;
    p->precision = precision;
    p->max_active = 1024;
    p->dt = 0.0025;
    ifl_batch_default_options(&p->batch);
}

int ifl_server_create(const ifl_server_params *p, ifl_server **out) {
    if (!p || !out) return IFL_ERR_ARG;
    *out = nullptr;
    if (p->variant < IFL_PLAIN || p->variant > IFL_VARDENS || (p->precision != IFL_FP64 && p->precision != IFL_FP32) ||
        p->device < 0 || p->max_active < 1 || !(p->dt > 0.0) || p->hbm_budget_bytes < 0)
        return IFL_ERR_ARG;
    if (!p->dry_run && cudaSetDevice(p->device) != cudaSuccess) {
        cudaGetLastError();
        return IFL_ERR_CUDA;
    }
    ifl_server *s = new (std::nothrow) ifl_server;
    if (!s) return IFL_ERR_NOMEM;
    try {
        s->impl = ifl::server_create(*p);
    } catch (...) {
        delete s;
        return IFL_ERR_NOMEM;
    }
    s->dry = p->dry_run != 0;
    *out = s;
    return IFL_OK;
}

int ifl_server_destroy(ifl_server *s) {
    if (!s) return IFL_ERR_ARG;
    if (!s->dry) cudaSetDevice(ifl::server_device(s->impl));
    delete s;
    return IFL_OK;
}

double ifl_server_now(const ifl_server *s) { return (s && s->impl) ? ifl::server_now(s->impl) : 0.0; }

int ifl_server_submit(ifl_server *s, const ifl_request *r, int64_t *id) {
    if (!r) return IFL_ERR_ARG;
    return sguarded(s, [&](ifl::Server *v) { return ifl::server_submit(v, *r, id); });
}

int ifl_server_step(ifl_server *s, int *active, int *queued) {
    return sguarded(s, [&](ifl::Server *v) { return ifl::server_step(v, active, queued); });
}

int ifl_server_completions(ifl_server *s, ifl_completion *out, int capacity, int *n) {
    if (capacity < 0 || (capacity > 0 && !out)) return IFL_ERR_ARG;
    return sguarded(s, [&](ifl::Server *v) { return ifl::server_completions(v, out, capacity, n); });
}

int ifl_server_read_field(ifl_server *s, int64_t id, int field, void *host, size_t bytes, int dtype) {
    return sguarded(s, [&](ifl::Server *v) { return ifl::server_read_field(v, id, field, host, bytes, dtype); });
}

int ifl_server_field_shape(ifl_server *s, int64_t id, int field, int *w, int *h) {
    return sguarded(s, [&](ifl::Server *v) { return ifl::server_field_shape(v, id, field, w, h); });
}

int ifl_server_request_stats(ifl_server *s, int64_t id, ifl_step_stats *out) {
    return sguarded(s, [&](ifl::Server *v) { return ifl::server_stats(v, id, out); });
}

int ifl_server_release(ifl_server *s, int64_t id) {
    return sguarded(s, [&](ifl::Server *v) { return ifl::server_release(v, id); });
}

int ifl_server_get_info(const ifl_server *s, ifl_server_info *out) {
    if (!s || !s->impl || !out) return IFL_ERR_ARG;
    ifl::server_info(s->impl, out);
    return IFL_OK;
}

const char *ifl_server_last_error(const ifl_server *s) {
    return (s && s->impl) ? ifl::server_error(s->impl).c_str() : "invalid server";
}

int64_t ifl_device_bytes(const ifl_params *p) {
    if (!p || p->w < 2 || p->h < 2 || p->w > 32768 || p->h > 32768 || p->variant < IFL_GS_EULER ||
        p->variant > IFL_FLIP || (p->precision != IFL_FP64 && p->precision != IFL_FP32))
        return IFL_ERR_ARG;
    int sms = 152, dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaGetLastError();
    return (int64_t)ifl::solver_device_bytes(*p, 2 * sms);
}

const char *ifl_version(void) { return "ifluids-gb300 0.2 (sm_103a)"; }

// ------------------------------------------------------------------ batches
void ifl_batch_default_options(ifl_batch_options *o) {
    if (!o) return;
    std::memset(o, 0, sizeof *o);
    o->use_graph = 1;
    o->tune_iterations = 8;
    o->tile_tune = 1;
    for (int p = 0; p < 8; p++) {
        o->tile_w[p] = 32;
        o->tile_h[p] = 8;
    }
}

int ifl_batch_create(ifl_solver *const *members, int n, const ifl_batch_options *opt, ifl_batch **out) {
    if (!members || n <= 0 || !out) return IFL_ERR_ARG;
    *out = nullptr;
    ifl_batch_options o;
    if (opt) o = *opt;
    else ifl_batch_default_options(&o);
    std::vector<ifl::SolverBase *> m(n);
    for (int i = 0; i < n; i++) {
        if (!members[i] || !members[i]->impl) return IFL_ERR_ARG;
        m[i] = members[i]->impl.get();
    }
    ifl_batch *b = new (std::nothrow) ifl_batch;
    if (!b) return IFL_ERR_NOMEM;
    if (m[0]->activate() != 0) {
        delete b;
        return IFL_ERR_CUDA;
    }
    std::string err;
    int e;
    try {
        e = ifl::make_batch(m.data(), n, o, &b->impl, &err);
    } catch (...) {
        e = IFL_ERR_NOMEM;
        err = "host allocation failed";
    }
    if (e != IFL_OK) {
        g_batch_create_error = err.empty() ? "invalid batch arguments" : err;
        delete b;
        return e;
    }
    *out = b;
    return IFL_OK;
}

int ifl_batch_destroy(ifl_batch *b) {
    if (!b) return IFL_ERR_ARG;
    if (b->impl) cudaSetDevice(b->impl->device());
    delete b;
    return IFL_OK;
}

int ifl_batch_set_inflows(ifl_batch *b, int member, const ifl_inflow *rects, int n) {
    return bguarded(b, [&](ifl::BatchBase &v) { return v.set_inflows(member, rects, n); });
}

int ifl_batch_update(ifl_batch *b, double dt) {
    return bguarded(b, [&](ifl::BatchBase &v) { return v.update(dt); });
}

int ifl_batch_get_stats(ifl_batch *b, ifl_step_stats *out, int n) {
    return bguarded(b, [&](ifl::BatchBase &v) { return v.get_stats(out, n); });
}

int ifl_batch_get_info(ifl_batch *b, ifl_batch_info *out) {
    if (!out) return IFL_ERR_ARG;
    return bguarded(b, [&](ifl::BatchBase &v) { return v.info(out); });
}

int ifl_batch_plan_teams(int grid, int strips_per_block, int n, const int *strips, const double *work,
                         int *teams) {
    if (grid <= 0 || strips_per_block <= 0 || n <= 0 || !strips || !work || !teams) return IFL_ERR_ARG;
    for (int i = 0; i < n; i++)
        if (strips[i] <= 0 || !(work[i] >= 0.0)) return IFL_ERR_ARG;
    try {
        int tsize[8];
        const int used = ifl::pcg_plan_teams(grid, strips_per_block, n, strips, work, nullptr, teams, tsize, nullptr);
        return used < 0 ? (int)IFL_ERR_UNSUPPORTED : used;
    } catch (...) {
        return IFL_ERR_NOMEM;
    }
}

void *ifl_batch_stream(ifl_batch *b) { return (b && b->impl) ? (void *)b->impl->stream() : nullptr; }

const char *ifl_batch_last_error(const ifl_batch *b) {
    if (!b) return g_batch_create_error.c_str();  // why the last ifl_batch_create on this thread failed
    return b->impl ? b->impl->error().c_str() : "invalid batch";
}

}  // extern "C"
