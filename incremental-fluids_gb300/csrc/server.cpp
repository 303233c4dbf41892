// server.cpp - continuous-batching request loop (ifl_server_*).
//
// Requests (a scene: grid size, bodies, inflow rectangles, number of update()
// calls) arrive at any time and wait in arrival order.  Before every step the
// loop admits waiting requests, first come first served, while their device
// state fits the HBM budget and the member cap; every admitted request then
// advances one update() in one batch step (batch.cu) together with all the
// others, so requests of different sizes that arrive while others run share
// the GPU from their first step on.  A request that has done its steps leaves
// the batch; its state stays on the device until the caller has read what it
// needs and releases it.  The batch is rebuilt whenever its membership
// changes, with the PCG launch shape the first batch's autotuner chose.
//
// A scene's arithmetic does not depend on the other members: the batched
// phases are per scene, and the PCG team that solves a scene has the size its
// strip count selects whatever else runs.  A request's results are therefore
// bit-identical alone and in any mix.
//
// dry_run: no device work at all (admission, queueing and latency bookkeeping
// only), for capacity planning and for testing the loop without a GPU.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <vector>

#include "solver.h"

namespace ifl {

namespace {

struct Request {
    int64_t id = 0;
    ifl_params prm{};
    std::vector<ifl_body> bodies;
    std::vector<ifl_inflow> inflows;
    int steps = 0, done = 0;
    double arrival = 0.0, admitted = -1.0, finished = -1.0;
    size_t bytes = 0;
    std::unique_ptr<SolverBase> solver;
    enum { QUEUED, ACTIVE, DONE } state = QUEUED;
};

}  // namespace

class Server {
  public:
    explicit Server(const ifl_server_params &p) : p_(p), t0_(std::chrono::steady_clock::now()) {
        int sms = 76 * 2;  // PCG partial sums are sized by the SM count
        if (!p_.dry_run) {
            int dev = 0;
            if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            cudaGetLastError();
        }
        max_blocks_ = 2 * sms;
        opt_ = p_.batch;
    }
    ~Server() {
        batch_.reset();
        reqs_.clear();
    }

    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
    }

    int submit(const ifl_request &r, int64_t *id) {
        if (r.w < 2 || r.h < 2 || r.w > 32768 || r.h > 32768 || r.steps < 1 || r.n_bodies < 0 || r.n_bodies > 256 ||
            r.n_inflows < 0 || r.n_inflows > 8 || (r.n_bodies && !r.bodies) || (r.n_inflows && !r.inflows))
            return IFL_ERR_ARG;
        for (int i = 0; i < r.n_bodies; i++)
            if (r.bodies[i].type != 0 && r.bodies[i].type != 1) return IFL_ERR_ARG;
        auto q = std::make_unique<Request>();
        q->id = next_id_++;
        ifl_default_params(&q->prm, p_.variant, r.w, r.h);
        q->prm.precision = p_.precision;
        q->prm.device = p_.device;
        q->bodies.assign(r.bodies, r.bodies + r.n_bodies);
        q->inflows.assign(r.inflows, r.inflows + r.n_inflows);
        q->steps = r.steps;
        q->arrival = r.arrival;
        q->bytes = solver_device_bytes(q->prm, max_blocks_);
        if (p_.hbm_budget_bytes > 0 && (int64_t)q->bytes > p_.hbm_budget_bytes) {
            err_ = "request larger than the whole HBM budget";
            return IFL_ERR_NOMEM;
        }
        if (id) *id = q->id;
        queue_.push_back(q.get());
        reqs_[q->id] = std::move(q);
        return IFL_OK;
    }

    int step(int *n_active, int *n_queued) {
        admit();
        peak_queued_ = std::max<int64_t>(peak_queued_, (int64_t)queue_.size());
        int e = IFL_OK;
        if (!active_.empty()) {
            if (!p_.dry_run) {
                const bool fresh = dirty_;
                const auto t0 = std::chrono::steady_clock::now();
                if (dirty_) {
                    if ((e = rebuild())) return e;
                }
                const auto t1 = std::chrono::steady_clock::now();
                if ((e = batch_->update(p_.dt))) {
                    err_ = batch_->error();
                    return e;
                }
                if (fresh) {
                    // a new membership: building the batch, plus what its first
                    // step spends beyond a steady step (plan, graph capture)
                    const auto t2 = std::chrono::steady_clock::now();
                    const double build = std::chrono::duration<double, std::milli>(t1 - t0).count();
                    const double first = std::chrono::duration<double, std::milli>(t2 - t1).count();
                    rebuild_ms_ += build + std::max(0.0, first - last_steady_ms_);
                } else {
                    last_steady_ms_ = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t1).count();
                }
            }
            const double t = now();
            steps_run_++;
            std::vector<Request *> still;
            for (Request *q : active_) {
                q->done++;
                cell_steps_ += (int64_t)q->prm.w * q->prm.h;
                if (!p_.dry_run) q->solver->advance_bodies(p_.dt);  // SolidBody::update between steps
                if (q->done >= q->steps) {
                    completed_++;
                    q->state = Request::DONE;
                    q->finished = t;
                    finished_.push_back(q->id);
                    dirty_ = true;
                } else {
                    still.push_back(q);
                }
            }
            active_.swap(still);
            if (dirty_) batch_.reset();  // members left: the next step builds a new batch
        }
        if (n_active) *n_active = (int)active_.size();
        if (n_queued) *n_queued = (int)queue_.size();
        return IFL_OK;
    }

    int completions(ifl_completion *out, int capacity, int *n) {
        int k = 0;
        while (k < capacity && !finished_.empty()) {
            const Request &q = *reqs_.at(finished_.front());
            finished_.pop_front();
            ifl_completion &c = out[k++];
            std::memset(&c, 0, sizeof c);
            c.id = q.id;
            c.w = q.prm.w;
            c.h = q.prm.h;
            c.steps = q.steps;
            c.arrival = q.arrival;
            c.admitted = q.admitted;
            c.finished = q.finished;
            c.device_bytes = (int64_t)q.bytes;
        }
        if (n) *n = k;
        return IFL_OK;
    }

    Request *find(int64_t id) {
        auto it = reqs_.find(id);
        return it == reqs_.end() ? nullptr : it->second.get();
    }

    int read_field(int64_t id, int field, void *host, size_t bytes, int dtype) {
        Request *q = find(id);
        if (!q || q->state == Request::QUEUED || !q->solver) return IFL_ERR_ARG;
        int e = q->solver->read_field(field, host, bytes, dtype);
        if (e) err_ = q->solver->error();
        return e;
    }

    int field_shape(int64_t id, int field, int *w, int *h) {
        Request *q = find(id);
        if (!q || !q->solver || !w || !h) return IFL_ERR_ARG;
        void *p;
        int elem, sd;
        return q->solver->field_info(field, &p, &elem, w, h, &sd);
    }

    int stats(int64_t id, ifl_step_stats *st) {
        Request *q = find(id);
        if (!q || !q->solver || !st) return IFL_ERR_ARG;
        return q->solver->read_pcg(st);
    }

    int release(int64_t id) {
        Request *q = find(id);
        if (!q || q->state != Request::DONE) return IFL_ERR_ARG;
        in_use_ -= q->bytes;
        reqs_.erase(id);
        return IFL_OK;
    }

    void info(ifl_server_info *o) const {
        std::memset(o, 0, sizeof *o);
        o->active = (int)active_.size();
        o->queued = (int)queue_.size();
        o->bytes_in_use = (int64_t)in_use_;
        o->cell_steps = cell_steps_;
        o->steps = steps_run_;
        o->rebuilds = rebuilds_;
        o->threads = opt_.threads;
        o->strips_per_block = opt_.strips_per_block;
        o->stages = opt_.stages;
        o->peak_queued = peak_queued_;
        o->admitted = admitted_;
        o->completed = completed_;
        o->rebuild_ms = rebuild_ms_;
    }

    const std::string &error() const { return err_; }
    void set_error(const std::string &e) { err_ = e; }
    int device() const { return p_.device; }

  private:
    // First come, first served: the head of the queue waits until it fits.
    void admit() {
        while (!queue_.empty()) {
            Request *q = queue_.front();
            if ((int)active_.size() >= p_.max_active) break;
            if (p_.hbm_budget_bytes > 0 && (int64_t)(in_use_ + q->bytes) > p_.hbm_budget_bytes) break;
            if (!p_.dry_run) {
                q->solver = make_solver(q->prm);
                int e = q->solver->init();
                if (e) {
                    // the device refused (fragmentation, other users): retry later
                    q->solver.reset();
                    break;
                }
                if (!q->bodies.empty()) q->solver->set_bodies(q->bodies.data(), (int)q->bodies.size());
            }
            queue_.pop_front();
            admitted_++;
            in_use_ += q->bytes;
            q->state = Request::ACTIVE;
            q->admitted = now();
            active_.push_back(q);
            dirty_ = true;
        }
    }

    int rebuild() {
        batch_.reset();
        std::vector<SolverBase *> m;
        for (Request *q : active_) m.push_back(q->solver.get());
        std::string why;
        int e = make_batch(m.data(), (int)m.size(), opt_, &batch_, &why);
        if (e) {
            err_ = "batch: " + why;
            return e;
        }
        for (size_t i = 0; i < active_.size(); i++) {
            Request *q = active_[i];
            if (int e2 = batch_->set_inflows((int)i, q->inflows.data(), (int)q->inflows.size())) return e2;
        }
        rebuilds_++;
        dirty_ = false;
        if (opt_.threads == 0 || opt_.tile_tune == 1) tune_pending_ = true;
        return IFL_OK;
    }

  public:
    // After the first step of an autotuned batch: keep its shape for later batches.
    void pin_shape() {
        if (!tune_pending_ || !batch_) return;
        ifl_batch_info bi;
        if (batch_->info(&bi) == IFL_OK && bi.threads > 0) {
            opt_.threads = bi.threads;
            opt_.strips_per_block = bi.strips_per_block;
            opt_.stages = bi.stages;
            // and its tile shapes: a rebuilt batch times no candidates again
            opt_.tile_tune = 2;
            for (int p = 0; p < 8; p++) {
                opt_.tile_w[p] = bi.tile_w[p];
                opt_.tile_h[p] = bi.tile_h[p];
            }
            tune_pending_ = false;
        }
    }

  private:
    ifl_server_params p_;
    ifl_batch_options opt_;
    std::chrono::steady_clock::time_point t0_;
    int max_blocks_ = 304;
    int64_t next_id_ = 1;
    std::map<int64_t, std::unique_ptr<Request>> reqs_;
    std::deque<Request *> queue_;
    std::vector<Request *> active_;
    std::deque<int64_t> finished_;
    std::unique_ptr<BatchBase> batch_;
    bool dirty_ = false, tune_pending_ = false;
    size_t in_use_ = 0;
    int64_t cell_steps_ = 0, steps_run_ = 0, rebuilds_ = 0, peak_queued_ = 0, admitted_ = 0, completed_ = 0;
    double rebuild_ms_ = 0.0, last_steady_ms_ = 0.0;
    std::string err_;
};

Server *server_create(const ifl_server_params &p) { return new Server(p); }
void server_destroy(Server *s) { delete s; }
double server_now(const Server *s) { return s->now(); }
int server_submit(Server *s, const ifl_request &r, int64_t *id) { return s->submit(r, id); }
int server_step(Server *s, int *a, int *q) {
    int e = s->step(a, q);
    if (e == IFL_OK) s->pin_shape();
    return e;
}
int server_completions(Server *s, ifl_completion *o, int cap, int *n) { return s->completions(o, cap, n); }
int server_read_field(Server *s, int64_t id, int field, void *host, size_t bytes, int dtype) {
    return s->read_field(id, field, host, bytes, dtype);
}
int server_stats(Server *s, int64_t id, ifl_step_stats *st) { return s->stats(id, st); }
int server_field_shape(Server *s, int64_t id, int field, int *w, int *h) { return s->field_shape(id, field, w, h); }
int server_release(Server *s, int64_t id) { return s->release(id); }
void server_info(const Server *s, ifl_server_info *o) { s->info(o); }
const std::string &server_error(const Server *s) { return s->error(); }
void server_set_error(Server *s, const std::string &e) { s->set_error(e); }
int server_device(const Server *s) { return s->device(); }

}  // namespace ifl
