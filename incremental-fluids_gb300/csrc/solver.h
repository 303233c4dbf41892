// solver.h - host-side solver object behind the C ABI.
#pragma once
#include <memory>
#include <string>
#include <vector>

#include "ifluids.h"
#include "ifl_internal.h"

namespace ifl {

class SolverBase {
  public:
    explicit SolverBase(const ifl_params &p) : prm_(p) {}
    virtual ~SolverBase() = default;

    virtual int init() = 0;
    virtual int add_inflow(double x, double y, double w, double h, double d, double t, double u, double v) = 0;
    virtual int update(double dt) = 0;
    virtual int run_phase(int phase, double dt) = 0;
    // *sd: 1 when the array is stored in the strip-diagonal layout (see SDIdx)
    virtual int field_info(int field, void **ptr, int *elem, int *w, int *h, int *sd) const = 0;
    virtual SDIdx sd_index() const = 0;
    virtual int flip(int q) = 0;
    virtual int read_pcg(ifl_step_stats *st) = 0;
    virtual size_t pitch() const = 0;
    virtual size_t device_bytes() const = 0;
    // toImage into a host buffer (synchronising) or a device buffer (async).
    virtual int render(int heat, void *rgba, size_t bytes, bool on_device) = 0;

    // Step 8 (FLIP) particle state; IFL_ERR_ARG for the other variants.
    virtual int particle_count(int *n) { (void)n; return IFL_ERR_ARG; }
    virtual int read_particles(int which, double *out, int capacity, int *n) {
        (void)which; (void)out; (void)capacity; (void)n;
        return IFL_ERR_ARG;
    }
    virtual int write_particles(int which, const double *in, int n) {
        (void)which; (void)in; (void)n;
        return IFL_ERR_ARG;
    }
    virtual int set_particle_count(int n) { (void)n; return IFL_ERR_ARG; }
    virtual int flip_init() { return IFL_ERR_ARG; }
    virtual int rng_state(uint32_t *get, const uint32_t *set) { (void)get; (void)set; return IFL_ERR_ARG; }

    // Access for the batch (batch.cu): Scene<F>* and PcgScratch* of this
    // handle, F as its precision.
    virtual void *scene_ptr() = 0;
    virtual void *scratch_ptr() = 0;
    virtual bool has_quantity(int q) const = 0;
    void count_step() { steps_++; }
    int pinned_pressure() const { return pinned_; }
    int pinned_heat() const { return pinned_heat_; }

    int set_bodies(const ifl_body *b, int n);
    int advance_bodies(double dt);
    const std::vector<ifl_body> &bodies() const { return bodies_; }
    int read_field(int field, void *host, size_t bytes, int dtype);
    int write_field(int field, const void *host, size_t bytes, int dtype);

    void set_pinned(int pressure, int heat) {
        pinned_ = pressure;
        pinned_heat_ = heat;
    }
    void set_wait_limit(long long polls) { wait_limit_ = polls; }
    long long wait_limit() const { return wait_limit_; }
    int set_timing(bool on);
    int get_timing(ifl_timing *out);
    virtual int read_iteration_total(long long *out) = 0;
    int activate() const { return cudaSetDevice(prm_.device) == cudaSuccess ? 0 : -1; }
    cudaStream_t stream() const { return stream_; }
    const ifl_params &params() const { return prm_; }
    int64_t launches() const { return launches_; }
    const std::string &error() const { return err_; }
    void set_error(const std::string &e) { err_ = e; }

  protected:
    bool check(cudaError_t e, const char *what);
    // Event bracketing of one kernel group (no-op unless timing is on).
    int tbegin(int group);
    void tend(int rec);
    void release_timing();

    struct TimedRec {
        int group;
        cudaEvent_t start, stop;
    };
    bool timing_on_ = false;
    std::vector<TimedRec> recs_;
    std::vector<cudaEvent_t> event_pool_;

    ifl_params prm_;
    cudaStream_t stream_ = nullptr;
    bool own_stream_ = false;
    std::vector<ifl_body> bodies_;
    bool bodies_dirty_ = false;
    int pinned_ = -1, pinned_heat_ = -1;
    long long wait_limit_ = 0;  // polls of one device-side wait; 0: the default (about a second)
    uint32_t steps_ = 0;
    int64_t launches_ = 0;
    std::string err_;
};

std::unique_ptr<SolverBase> make_solver(const ifl_params &p);
// Device bytes a handle of these parameters allocates (max_blocks: PCG partial
// sums per scene, 2 x the SM count on the device).
size_t solver_device_bytes(const ifl_params &p, int max_blocks);

// Host-side conversion of a body to its device record (trigonometry by the C library).
void to_dev_body(const ifl_body &b, DevBody &d);

// A batch of handles stepped together (batch.cu).
class BatchBase {
  public:
    virtual ~BatchBase() = default;
    virtual int set_inflows(int member, const ifl_inflow *rects, int n) = 0;
    virtual int update(double dt) = 0;
    virtual int get_stats(ifl_step_stats *out, int n) = 0;
    virtual int info(ifl_batch_info *out) = 0;
    virtual cudaStream_t stream() const = 0;
    virtual int device() const = 0;
    const std::string &error() const { return err_; }
    void set_error(const std::string &e) { err_ = e; }

  protected:
    std::string err_;
};

// Continuous-batching request loop (server.cpp).
class Server;
Server *server_create(const ifl_server_params &p);
void server_destroy(Server *s);
double server_now(const Server *s);
int server_submit(Server *s, const ifl_request &r, int64_t *id);
int server_step(Server *s, int *active, int *queued);
int server_completions(Server *s, ifl_completion *out, int capacity, int *n);
int server_read_field(Server *s, int64_t id, int field, void *host, size_t bytes, int dtype);
int server_stats(Server *s, int64_t id, ifl_step_stats *st);
int server_field_shape(Server *s, int64_t id, int field, int *w, int *h);
int server_release(Server *s, int64_t id);
void server_info(const Server *s, ifl_server_info *out);
const std::string &server_error(const Server *s);
void server_set_error(Server *s, const std::string &e);
int server_device(const Server *s);

// Validates the members (one device, variant and precision) and builds the batch.
int make_batch(SolverBase *const *members, int n, const ifl_batch_options &opt, std::unique_ptr<BatchBase> *out,
               std::string *err);

}  // namespace ifl
