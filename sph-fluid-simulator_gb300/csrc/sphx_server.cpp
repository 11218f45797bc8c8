// Served form: a continuous-batching request loop over one resident batch.
//
// Requests (a scene plus a step count) are copied in at submission.  A worker
// thread admits queued requests in arrival order while their device
// footprint fits the HBM budget, lays the live scenes out as one batch
// (scenes already running keep their device state and move device to device;
// new ones are uploaded), advances every live scene together by up to
// steps_per_tick steps, retires each scene the moment it reaches its step
// count (results copied to host) and repeats.  Requests that arrive while
// others run join at the next tick; their work overlaps on the device.
// A scene's result does not depend on what else runs beside it: the batch
// kernels treat scenes independently and walk each in the same order as a
// handle holding that scene alone.
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "sphx_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t ticket;
    sphx_settings s;
    sphx_box box;
    uint32_t n;
    int nsteps;
    int steps_done = 0;
    int state = SPHX_REQ_QUEUED;
    int error = 0;
    size_t bytes = 0;
    std::vector<float> pos, vel;  // inputs, then results
    std::vector<float> rho, prs;
    double submit_s = 0, admit_s = 0, done_s = 0;
};

// Device bytes a scene needs in the batch: the per-particle arrays of the
// arena plus its cell-grid slots (counts and starts), as laid out by
// sphx_api.cpp, with the grid estimated from the particle count.
size_t footprint(uint32_t n) {
    // state, ids, records, sort scratch, staging, neighbour records and lists,
    // deferred-particle lists
    const size_t per_particle =
        16 * 4 + 4 * 2 + 16 + 16 + 4 * 3 + 8 + 24 + 32 + 4 * sphx::kNbrSlotsDefault + 4 + 9;
    // counts, starts, row offsets (at most one per slot), cell flags
    const size_t slots = 16ull * n + 4096;
    return per_particle * n + 13 * slots + 4096;
}

}  // namespace

struct sphx_server {
    sphx_server_options opt{};
    std::mutex mu;
    std::condition_variable cv, done_cv;
    std::deque<Request *> queue;            // submitted, not admitted
    std::map<uint64_t, Request *> all;      // every request not yet collected
    std::vector<Request *> live;            // in the batch, batch order
    uint64_t next_ticket = 1;
    size_t bytes_in_use = 0;
    bool stop = false;
    int inject = 0;  // host-side fault injection: the next tick fails with this code
    int fatal = 0;
    std::string fatal_msg;
    sphx_handle *h = nullptr;
    Clock::time_point t0;
    sphx_server_stats stats{};
    std::thread worker;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
    void run();
};

void sphx_server::run() {
    cudaSetDevice(opt.device);
    std::unique_lock<std::mutex> lock(mu);
    while (!stop) {
        // Admission, in arrival order, by HBM budget and scene limit.
        std::vector<Request *> admitted;
        while (!queue.empty()) {
            Request *r = queue.front();
            const bool fits = bytes_in_use + r->bytes <= opt.hbm_budget_bytes;
            const bool room = opt.max_scenes <= 0 || (int)(live.size() + admitted.size()) < opt.max_scenes;
            if (!(fits && room) && !(live.empty() && admitted.empty())) break;  // a lone request always runs
            queue.pop_front();
            bytes_in_use += r->bytes;
            r->state = SPHX_REQ_RUNNING;
            r->admit_s = now();
            admitted.push_back(r);
        }
        if (live.empty() && admitted.empty()) {
            cv.wait_for(lock, std::chrono::milliseconds(1));
            continue;
        }
        lock.unlock();
        int rc = SPHX_OK;
        // where the tick's time goes: laying scenes out, stepping, reading
        // finished scenes back (added to the stats under the lock below)
        double t_layout = 0, t_step = 0, t_read = 0;
        uint64_t n_layouts = 0, n_steps = 0;
        auto t = Clock::now();
        auto lap = [&](double &acc) {
            const auto now = Clock::now();
            acc += std::chrono::duration<double>(now - t).count();
            t = now;
        };
        if (!admitted.empty()) {
            std::vector<sphx::SceneInit> inits;
            for (size_t k = 0; k < live.size(); ++k) {
                sphx::SceneInit in{};
                in.keep = (int)k;
                inits.push_back(in);
            }
            for (Request *r : admitted) {
                sphx::SceneInit in{};
                in.s = r->s;
                in.box = r->box;
                in.n = r->n;
                in.pos3 = r->pos.data();
                in.vel3 = r->vel.empty() ? nullptr : r->vel.data();
                in.keep = -1;
                inits.push_back(in);
            }
            if (!h) {
                sphx_options o;
                sphx_options_default(&o);
                o.device = opt.device;
                rc = sphx::create_handle(inits.data(), inits.size(), &o, &h);
            } else {
                rc = sphx::relayout(h, inits);
            }
            for (Request *r : admitted) live.push_back(r);
            n_layouts += 1;
            lap(t_layout);
        }
        // One tick: every live scene advances by the same number of steps.
        int k = opt.steps_per_tick;
        for (Request *r : live) k = std::min(k, r->nsteps - r->steps_done);
        {
            std::lock_guard<std::mutex> g(mu);
            if (inject) {
                rc = sphx::fail(inject, "injected failure");
                inject = 0;
            }
        }
        if (rc == SPHX_OK && k > 0) rc = sphx::run_steps(h, opt.dt, k);
        if (rc == SPHX_OK) rc = sphx::read_status(h);
        lap(t_step);
        std::vector<int> finished;
        if (rc == SPHX_OK) {
            n_steps = (uint64_t)h->n * (uint64_t)k;
            for (size_t j = 0; j < live.size(); ++j) {
                Request *r = live[j];
                r->steps_done += k;
                if (r->steps_done >= r->nsteps) {
                    r->pos.assign(3ull * r->n, 0.f);
                    r->vel.assign(3ull * r->n, 0.f);
                    r->rho.assign(r->n, 0.f);
                    r->prs.assign(r->n, 0.f);
                    rc = sphx::read_scene(h, j, r->pos.data(), r->vel.data(), r->rho.data(),
                                          r->prs.data(), nullptr);
                    if (rc) break;
                    finished.push_back((int)j);
                }
            }
        }
        lap(t_read);
        if (rc == SPHX_OK && !finished.empty()) {
            std::vector<sphx::SceneInit> inits;
            size_t f = 0;
            for (size_t j = 0; j < live.size(); ++j) {
                if (f < finished.size() && finished[f] == (int)j) {
                    ++f;
                    continue;
                }
                sphx::SceneInit in{};
                in.keep = (int)j;
                inits.push_back(in);
            }
            rc = sphx::relayout(h, inits);
            n_layouts += 1;
            lap(t_layout);
        }
        lock.lock();
        stats.relayouts += n_layouts;
        stats.layout_s += t_layout;
        stats.step_s += t_step;
        stats.readout_s += t_read;
        if (rc == SPHX_OK) {
            stats.ticks += 1;
            stats.particle_steps += n_steps;
        }
        if (rc != SPHX_OK) {
            fatal = rc;
            fatal_msg = sphx_last_error();
            // the batch is gone: every request not yet done fails with the
            // server's error, the queued ones too (nothing will admit them)
            for (Request *r : live) {
                r->state = SPHX_REQ_FAILED;
                r->error = rc;
            }
            for (Request *r : queue) {
                r->state = SPHX_REQ_FAILED;
                r->error = rc;
            }
            live.clear();
            queue.clear();
            stats.live_scenes = 0;
            stats.queued = 0;
            done_cv.notify_all();
            break;
        }
        if (!finished.empty()) {
            std::vector<Request *> keep;
            size_t f = 0;
            const double t_done = now();
            for (size_t j = 0; j < live.size(); ++j) {
                if (f < finished.size() && finished[f] == (int)j) {
                    ++f;
                    Request *r = live[j];
                    r->state = SPHX_REQ_DONE;
                    r->done_s = t_done;
                    bytes_in_use -= r->bytes;
                    stats.completed += 1;
                } else {
                    keep.push_back(live[j]);
                }
            }
            live.swap(keep);
            done_cv.notify_all();
        }
        stats.live_scenes = live.size();
        stats.queued = queue.size();
        stats.bytes_in_use = bytes_in_use;
    }
}

extern "C" {

void sphx_server_options_default(sphx_server_options *o) {
    if (!o) return;
    o->hbm_budget_bytes = 150ull * 1000 * 1000 * 1000;
    o->steps_per_tick = 10;
    o->max_scenes = 0;
    o->dt = 0.002f;
    o->device = 0;
}

int sphx_server_create(const sphx_server_options *opt, sphx_server **out) {
    using sphx::fail;
    if (!out) return fail(SPHX_ERR_INVALID, "null argument");
    sphx_server *s = new sphx_server();
    if (opt) s->opt = *opt;
    else sphx_server_options_default(&s->opt);
    if (s->opt.steps_per_tick < 1 || !(s->opt.dt > 0.f) || s->opt.hbm_budget_bytes == 0) {
        delete s;
        return fail(SPHX_ERR_INVALID, "server options: steps_per_tick >= 1, dt > 0, budget > 0");
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || s->opt.device < 0 || s->opt.device >= ndev) {
        cudaGetLastError();
        delete s;
        return fail(SPHX_ERR_CUDA, "no such CUDA device");
    }
    s->t0 = Clock::now();
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return SPHX_OK;
}

int sphx_server_submit(sphx_server *s, const sphx_request *q, uint64_t *ticket) {
    using sphx::fail;
    if (!s || !q || !q->pos3 || !ticket) return fail(SPHX_ERR_INVALID, "null argument");
    if (q->n == 0 || q->n >= (size_t)1 << 31 || q->nsteps < 1)
        return fail(SPHX_ERR_INVALID, "request needs particles and at least one step");
    Request *r = new Request();
    r->s = q->settings;
    r->box = q->box;
    r->n = (uint32_t)q->n;
    r->nsteps = q->nsteps;
    r->pos.assign(q->pos3, q->pos3 + 3 * q->n);
    if (q->vel3) r->vel.assign(q->vel3, q->vel3 + 3 * q->n);
    r->bytes = footprint(r->n);
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->fatal) {
        delete r;
        return fail(s->fatal, "server stopped: " + s->fatal_msg);
    }
    r->ticket = s->next_ticket++;
    r->submit_s = s->now();
    s->all[r->ticket] = r;
    s->queue.push_back(r);
    s->stats.submitted += 1;
    *ticket = r->ticket;
    s->cv.notify_one();
    return SPHX_OK;
}

int sphx_server_status(sphx_server *s, uint64_t ticket, sphx_request_status *out) {
    using sphx::fail;
    if (!s || !out) return fail(SPHX_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return fail(SPHX_ERR_INVALID, "unknown ticket");
    const Request *r = it->second;
    out->state = r->state;
    out->steps_done = r->steps_done;
    out->submit_s = r->submit_s;
    out->admit_s = r->admit_s;
    out->done_s = r->done_s;
    return SPHX_OK;
}

int sphx_server_wait(sphx_server *s, uint64_t ticket, double timeout_s) {
    using sphx::fail;
    if (!s) return fail(SPHX_ERR_INVALID, "null argument");
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return fail(SPHX_ERR_INVALID, "unknown ticket");
    Request *r = it->second;
    const auto until = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                          std::chrono::duration<double>(timeout_s));
    while (r->state == SPHX_REQ_QUEUED || r->state == SPHX_REQ_RUNNING) {
        if (s->done_cv.wait_until(lock, until) == std::cv_status::timeout &&
            (r->state == SPHX_REQ_QUEUED || r->state == SPHX_REQ_RUNNING))
            return fail(SPHX_ERR_STATE, "request not finished within the timeout");
    }
    if (r->state == SPHX_REQ_FAILED) return fail(r->error, "request failed: " + s->fatal_msg);
    return SPHX_OK;
}

int sphx_server_result(sphx_server *s, uint64_t ticket, float *pos3, float *vel3, float *rho,
                       float *prs) {
    using sphx::fail;
    if (!s) return fail(SPHX_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return fail(SPHX_ERR_INVALID, "unknown ticket");
    Request *r = it->second;
    if (r->state != SPHX_REQ_DONE) return fail(SPHX_ERR_STATE, "request not finished");
    const size_t n = r->n;
    if (pos3) std::copy(r->pos.begin(), r->pos.end(), pos3);
    if (vel3) std::copy(r->vel.begin(), r->vel.begin() + 3 * n, vel3);
    if (rho) std::copy(r->rho.begin(), r->rho.end(), rho);
    if (prs) std::copy(r->prs.begin(), r->prs.end(), prs);
    s->all.erase(it);
    delete r;
    return SPHX_OK;
}

int sphx_server_inject_failure(sphx_server *s, int code) {
    using sphx::fail;
    if (!s || code >= 0) return fail(SPHX_ERR_INVALID, "a server and a negative status code");
    std::lock_guard<std::mutex> lock(s->mu);
    s->inject = code;
    return SPHX_OK;
}

int sphx_server_stats_get(sphx_server *s, sphx_server_stats *out) {
    using sphx::fail;
    if (!s || !out) return fail(SPHX_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lock(s->mu);
    *out = s->stats;
    out->elapsed_s = s->now();
    return s->fatal ? fail(s->fatal, "server stopped: " + s->fatal_msg) : SPHX_OK;
}

int sphx_server_destroy(sphx_server *s) {
    if (!s) return SPHX_OK;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop = true;
        s->cv.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    if (s->h) sphx_destroy(s->h);
    for (auto &kv : s->all) delete kv.second;
    delete s;
    return SPHX_OK;
}

}  // extern "C"
