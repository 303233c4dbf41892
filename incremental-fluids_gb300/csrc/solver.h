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

    int set_bodies(const ifl_body *b, int n);
    int advance_bodies(double dt);
    const std::vector<ifl_body> &bodies() const { return bodies_; }
    int read_field(int field, void *host, size_t bytes, int dtype);
    int write_field(int field, const void *host, size_t bytes, int dtype);

    void set_pinned(int pressure, int heat) {
        pinned_ = pressure;
        pinned_heat_ = heat;
    }
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
    uint32_t steps_ = 0;
    int64_t launches_ = 0;
    std::string err_;
};

std::unique_ptr<SolverBase> make_solver(const ifl_params &p);

}  // namespace ifl
